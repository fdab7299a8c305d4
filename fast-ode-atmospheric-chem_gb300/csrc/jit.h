// The per-mechanism module of the generated variant (jit.cpp).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "device.cuh"
#include "fastode_gb300.h"
#include "symbolic.h"

namespace fo {

struct GenModule;

// Generate, link (or take from the cache in cache_dir; null: the default
// cache, empty: none) and load the module of a plan's tables.
int gen_create(const HostTables& t, const char* cache_dir, GenModule** out, fo_gen_info* info, std::string* err);
void gen_destroy(GenModule* m);
// Generate (and, with do_link, link) without a device: no module is loaded.
int gen_check(const HostTables& t, bool do_link, fo_gen_info* info, std::string* err);
// One launch of the generated integrator kernel: grid blocks of 32 lanes.
cudaError_t gen_launch(GenModule* m, const SolveParams& p, int grid, size_t smem, cudaStream_t stream);

}  // namespace fo
