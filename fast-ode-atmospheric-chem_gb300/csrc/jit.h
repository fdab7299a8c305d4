// The per-mechanism module of the generated variant (jit.cpp).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "codegen.h"
#include "device.cuh"
#include "fastode_gb300.h"
#include "symbolic.h"

namespace fo {

struct GenModule;

// Generate, link (or take from the cache in cache_dir; null: the default
// cache, empty: none) and load the module of one or several plans' tables
// (mechanism index = position in ts).
int gen_create(const std::vector<const HostTables*>& ts, const std::vector<GenOptions>& opts, const char* cache_dir,
               GenModule** out, fo_gen_info* info, std::string* err);
void gen_destroy(GenModule* m);
// Generate (and, with do_link, link) without a device: no module is loaded.
int gen_check(const HostTables& t, const GenOptions& opt, bool do_link, fo_gen_info* info, std::string* err);
// One launch of the generated integrator kernel: grid blocks of 32 lanes.
cudaError_t gen_launch(GenModule* m, const SolveParams& p, int grid, size_t smem, cudaStream_t stream);
// One launch of the generated adjoint kernel (fo_adjoint_interval): grid
// blocks of 32 lanes.
cudaError_t gen_launch_adjoint(GenModule* m, const AdjParams& a, int grid, size_t smem, cudaStream_t stream);
// One persistent launch of the generated several-mechanism kernel (the
// module made from every batch's tables, each batch's gen_index set); a
// cooperative launch when the batches run in lockstep rounds.
cudaError_t gen_launch_multi(GenModule* m, const SolveParams* batches, int nb, const int32_t* starts,
                             int32_t* queue, double* scratch, int64_t slot_doubles, int grid, size_t smem,
                             bool cooperative, cudaStream_t stream);
// Whether `grid` blocks of the single-batch (multi false) or several-mechanism
// kernel are all resident at once on the current device.
bool gen_resident(GenModule* m, bool multi, int grid, size_t smem);

}  // namespace fo
