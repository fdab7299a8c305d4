// Accuracy scores and the TS1 scenario's photolysis patch on the device.
//
// fo_score_accumulate: the sums behind Sandu's digits (fastode/ts1.py:226-264,
// fastode/reference.py:41-59) for one snapshot, one block per reference
// column, reduced in a fixed order so that repeated runs give the same bits;
// plus the sign/finiteness gate of the snapshot.
// fo_scale_photolysis: the per-interval photolysis columns of run_scenario
// (fastode/ts1.py:204-214).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "fastode_gb300.h"

namespace fo {
int set_last_error(int code, const char* what);
}

namespace {

constexpr int kScoreThreads = 256;

// Per column j: sum over cells of ((Y - ref) / ref)^2 and the number of
// cells counted. Rule FO_SCORE_TS1 skips ref < threshold (a NaN reference
// is counted); FO_SCORE_DIGITS keeps ref >= threshold (a NaN is not).
__global__ void __launch_bounds__(kScoreThreads)
score_columns_kernel(int C, const double* __restrict__ Y, int64_t ycs, int64_t yss, const int32_t* __restrict__ species,
                     const double* __restrict__ ref, int64_t rcs, int64_t rjs, double threshold, int rule,
                     double* __restrict__ sums, long long* __restrict__ counts) {
  __shared__ double s_acc[kScoreThreads / 32];
  __shared__ long long s_cnt[kScoreThreads / 32];
  const int j = blockIdx.x;
  const int sp = species[j];
  if (sp < 0) return;
  double acc = 0.0;
  long long cnt = 0;
  for (int c = threadIdx.x; c < C; c += blockDim.x) {
    const double r = ref[(int64_t)c * rcs + (int64_t)j * rjs];
    const bool keep = rule == FO_SCORE_TS1 ? !(r < threshold) : (r >= threshold);
    if (keep) {
      const double d = __ddiv_rn(__dsub_rn(Y[(int64_t)c * ycs + (int64_t)sp * yss], r), r);
      acc = __dadd_rn(acc, __dmul_rn(d, d));
      ++cnt;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    acc = __dadd_rn(acc, __shfl_down_sync(0xffffffffu, acc, off));
    cnt += __shfl_down_sync(0xffffffffu, cnt, off);
  }
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_acc[warp] = acc;
    s_cnt[warp] = cnt;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    long long k = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a = __dadd_rn(a, s_acc[w]);
      k += s_cnt[w];
    }
    sums[j] = __dadd_rn(sums[j], a);
    counts[j] += k;
  }
}

// gate = 0 when a value of the snapshot is non-finite or below -1e-20
// (fastode/ts1.py:240-241). Every writer writes the same 0.
__global__ void gate_kernel(int C, int n, const double* __restrict__ Y, int64_t ycs, int64_t yss, int32_t* gate) {
  const int64_t total = (int64_t)C * n;
  bool ok = true;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = e / C, c = e - s * C;
    const double v = Y[c * ycs + s * yss];
    if (!isfinite(v) || v < -1.0e-20) ok = false;
  }
  if (!__all_sync(0xffffffffu, ok) && (threadIdx.x & 31) == 0) *gate = 0;
}

// k(c, rxn[p]) = (base(p, c) * factor) * scaling[p]: the reference first sets
// params[name] = base * f and then k[:, j] = params[name] * scaling.
__global__ void scale_photolysis_kernel(int C, int nphoto, const int32_t* __restrict__ rxn,
                                        const double* __restrict__ base, const double* __restrict__ scaling,
                                        double factor, double* __restrict__ k, int64_t kcs, int64_t krs) {
  const int64_t total = (int64_t)C * nphoto;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(e / C);
    const int64_t c = e - (int64_t)p * C;
    k[c * kcs + (int64_t)rxn[p] * krs] = __dmul_rn(__dmul_rn(base[e], factor), scaling[p]);
  }
}

int grid_for(int64_t total, int block) {
  int64_t g = (total + block - 1) / block;
  const int64_t cap = 152 * 16;
  if (g > cap) g = cap;
  return (int)(g > 0 ? g : 1);
}

int launched(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fo::set_last_error(FO_E_CUDA, what);
  return FO_OK;
}

}  // namespace

extern "C" {

int fo_score_accumulate(int32_t C, int32_t n, const double* Y, int64_t y_cell_stride, int64_t y_species_stride,
                        int32_t m, const int32_t* species, const double* ref, int64_t ref_cell_stride,
                        int64_t ref_column_stride, double threshold, int32_t rule, double* sums, int64_t* counts,
                        int32_t* gate, void* stream) {
  if (C < 0 || n < 0 || m < 0) return fo::set_last_error(FO_E_INVALID, "negative size");
  if (rule != FO_SCORE_TS1 && rule != FO_SCORE_DIGITS) return fo::set_last_error(FO_E_INVALID, "unknown rule");
  if (C == 0) return FO_OK;
  if (!Y) return fo::set_last_error(FO_E_INVALID, "null argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (m > 0) {
    if (!species || !ref || !sums || !counts) return fo::set_last_error(FO_E_INVALID, "null argument");
    score_columns_kernel<<<m, kScoreThreads, 0, s>>>(C, Y, y_cell_stride, y_species_stride, species, ref,
                                                     ref_cell_stride, ref_column_stride, threshold, rule, sums,
                                                     reinterpret_cast<long long*>(counts));
    int rc = launched("score_columns_kernel");
    if (rc != FO_OK) return rc;
  }
  if (gate && n > 0) {
    gate_kernel<<<grid_for((int64_t)C * n, 256), 256, 0, s>>>(C, n, Y, y_cell_stride, y_species_stride, gate);
    return launched("gate_kernel");
  }
  return FO_OK;
}

int fo_scale_photolysis(int32_t C, int32_t nphoto, const int32_t* rxn, const double* base, const double* scaling,
                        double factor, double* k, int64_t k_cell_stride, int64_t k_reaction_stride, void* stream) {
  if (C < 0 || nphoto < 0) return fo::set_last_error(FO_E_INVALID, "negative size");
  if (C == 0 || nphoto == 0) return FO_OK;
  if (!rxn || !base || !scaling || !k) return fo::set_last_error(FO_E_INVALID, "null argument");
  scale_photolysis_kernel<<<grid_for((int64_t)C * nphoto, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      C, nphoto, rxn, base, scaling, factor, k, k_cell_stride, k_reaction_stride);
  return launched("scale_photolysis_kernel");
}

}  // extern "C"
