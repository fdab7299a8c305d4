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
// fo_rate_laws: every rate constant of a TS1-style mechanism (Arrhenius,
// Troe, user-defined and surface rows, the third-body fold) on the device.
// fo_fp64_fma_rate: a DFMA throughput kernel that states the FP64 roofline
// denominator on the device the integrator runs on.
#include <cuda_runtime.h>
#include <math_constants.h>

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

// The universal gas constant as the reference forms it (fastode/ts1.py:30-32)
// and pi as Python's math.pi.
constexpr double kBoltzmann = 1.380649e-23;
constexpr double kAvogadro = 6.02214076e23;
constexpr double kRGas = kBoltzmann * kAvogadro;
constexpr double kPi = 3.141592653589793;

// x ** e for an array x and a scalar e, as NumPy evaluates it: -1, 0, 0.5, 1
// and 2 by the reciprocal, one, the square root, x and the square; other
// exponents by pow.
__device__ double scalar_power(double x, double e) {
  if (e == 1.0) return x;
  if (e == -1.0) return __ddiv_rn(1.0, x);
  if (e == 0.0) return 1.0;
  if (e == 0.5) return __dsqrt_rn(x);
  if (e == 2.0) return __dmul_rn(x, x);
  return pow(x, e);
}

// One rate constant per thread, cells fastest (fastode/ts1.py:66-103, each
// expression in the reference's order, no contraction).
__global__ void rate_laws_kernel(int C, int R, const fo_rate_law* __restrict__ laws, const double* __restrict__ T,
                                 const double* __restrict__ P, const double* __restrict__ params, int64_t pcs,
                                 const double* __restrict__ power, double* __restrict__ k, int64_t kcs,
                                 int64_t krs) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)C * R) return;
  const int c = (int)(idx % C);
  const int j = (int)(idx / C);
  const fo_rate_law& L = laws[j];
  const double t = T[c], p = P[c];
  double v;
  switch (L.type) {
    case FO_RATE_ARRHENIUS:
      v = __dmul_rn(__dmul_rn(__dmul_rn(L.c[0], exp(__ddiv_rn(L.c[2], t))), scalar_power(__ddiv_rn(t, L.c[3]), L.c[1])),
                    __dadd_rn(1.0, __dmul_rn(L.c[4], p)));
      break;
    case FO_RATE_TROE: {
      const double M = __ddiv_rn(p, __dmul_rn(kRGas, t));
      const double k0 = __dmul_rn(__dmul_rn(L.c[0], exp(__ddiv_rn(L.c[2], t))), scalar_power(__ddiv_rn(t, 300.0), L.c[1]));
      const double kinf =
          __dmul_rn(__dmul_rn(L.c[3], exp(__ddiv_rn(L.c[5], t))), scalar_power(__ddiv_rn(t, 300.0), L.c[4]));
      const double k0M = __dmul_rn(k0, M);
      const double ratio = __ddiv_rn(k0M, kinf);
      const double l = log10(ratio);
      v = __dmul_rn(__ddiv_rn(k0M, __dadd_rn(1.0, ratio)), pow(L.c[6], __ddiv_rn(L.c[7], __dadd_rn(L.c[7], __dmul_rn(l, l)))));
      break;
    }
    case FO_RATE_USER:
      v = __dmul_rn(params[(int64_t)L.column * pcs + c], L.c[0]);
      break;
    case FO_RATE_SURFACE: {
      const double radius = params[(int64_t)L.column * pcs + c];
      const double number = params[(int64_t)(L.column + 1) * pcs + c];
      const double speed = __dsqrt_rn(__dmul_rn(L.c[0], t));
      const double num = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(4.0, number), kPi), radius), radius);
      v = __ddiv_rn(num, __dadd_rn(__ddiv_rn(radius, L.c[1]), __ddiv_rn(4.0, __dmul_rn(speed, L.c[2]))));
      break;
    }
    default:
      v = CUDART_NAN;
  }
  if (power != nullptr && power[j] != 0.0) {
    const double M = __ddiv_rn(p, __dmul_rn(kRGas, t));
    const double e = power[j];
    // M ** power with an array exponent: pow, exact for the exponents 1 and 2
    v = __dmul_rn(v, e == 1.0 ? M : (e == 2.0 ? __dmul_rn(M, M) : pow(M, e)));
  }
  k[(int64_t)c * kcs + (int64_t)j * krs] = v;
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

int fo_rate_laws(int32_t C, int32_t R, const fo_rate_law* laws, const double* T, const double* P,
                 const double* params, int64_t param_column_stride, const double* power, double* k,
                 int64_t k_cell_stride, int64_t k_reaction_stride, void* stream) {
  if (C < 0 || R < 0) return FO_E_INVALID;
  const int64_t total = (int64_t)C * R;
  if (total == 0) return FO_OK;
  if (!laws || !T || !P || !k) return FO_E_INVALID;
  const int block = 256;
  rate_laws_kernel<<<(unsigned)((total + block - 1) / block), block, 0, (cudaStream_t)stream>>>(
      C, R, laws, T, P, params, param_column_stride, power, k, k_cell_stride, k_reaction_stride);
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
