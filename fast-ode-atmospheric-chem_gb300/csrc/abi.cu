// The C-ABI: plans, workspace sizing and launches. Every entry point returns
// an FO_* code and never aborts; CUDA failures are reported with FO_E_CUDA
// and the text of the error is kept for fo_last_error().
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "device.cuh"
#include "fastode_gb300.h"
#include "jit.h"
#include "layout.h"
#include "symbolic.h"

namespace fo {
cudaError_t launch_solve(const SolveParams& p, int grid, size_t smem, cudaStream_t stream);
cudaError_t launch_eval(const SolveParams& p, int C, int want_jac, double* out, cudaStream_t stream);
cudaError_t launch_adjoint(const AdjParams& a, int grid, int lanes, size_t smem, cudaStream_t stream);
int set_last_error(int code, const char* what);
cudaError_t launch_solve_multi(const SolveParams* batches, int nb, const int32_t* starts, int32_t* queue,
                               double* scratch, int64_t slot_doubles, int grid, int lanes, size_t smem,
                               cudaStream_t stream);
}  // namespace fo

struct fo_plan {
  fo::HostTables host;
  fo::DevTables dev;
  void* blob = nullptr;  // device copy of every table
  int device = -1;
  fo::GenModule* gen = nullptr;  // the generated variant's module (fo_plan_generate)
  fo::GenOptions gen_options;    // its register tile and solve block (fo_plan_set_generation)
  fo_gen_info gen_info{};
  std::mutex gen_mutex;
};

namespace {

thread_local std::string g_last_error = "";

int fail(int code, const std::string& what) {
  g_last_error = what;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return FO_E_CUDA;
}

}  // namespace

// Error text for the other translation units of the library.
int fo::set_last_error(int code, const char* what) { return fail(code, what); }

namespace {

using fo::layout_of;

const fo::DevTableau kTableaus[2] = {
    // ROS3 (fastode/tableaus.py:70-80)
    {0.43586652150845899941601945119356,
     3,
     {{0, 0, 0, 0}, {1.0, 0, 0, 0}, {1.0, 0.0, 0, 0}, {0, 0, 0, 0}},
     {{0, 0, 0, 0},
      {-0.10156171083877702091975600115545e01, 0, 0, 0},
      {0.40759956452537699824805835358067e01, 0.92076794298330791242156818474003e01, 0, 0},
      {0, 0, 0, 0}},
     {1.0, 0.61697947043828245592553615689730e01, -0.42772256543218573326238373806514, 0},
     {0.5, -0.29079558716805469821718236208017e01, 0.22354069897811569627360909276199, 0},
     {1, 1, 0, 0}},
    // RODAS3 (fastode/tableaus.py:82-90)
    {0.5,
     4,
     {{0, 0, 0, 0}, {0.0, 0, 0, 0}, {2.0, 0.0, 0, 0}, {2.0, 0.0, 1.0, 0}},
     {{0, 0, 0, 0}, {4.0, 0, 0, 0}, {1.0, -1.0, 0, 0}, {1.0, -1.0, -8.0 / 3.0, 0}},
     {2.0, 0.0, 1.0, 1.0},
     {0.0, 0.0, 0.0, 1.0},
     {1, 0, 1, 1}},
};

int lanes_for(int cells) { return ((cells + 31) / 32) * 32; }

// Shared-memory items per lane: the solve vector (n), or the compressed work
// row plus the prefetch ring of the pipelined factorization, whichever is
// larger (the two phases never overlap).
int region_items(const fo::HostTables& t) {
  const int ring = fo::kRingChunks * fo::kStreamChunk;
  return t.n > t.max_row_len + ring ? t.n : t.max_row_len + ring;
}

// The compact variant's items per lane: half a row and its ring, or half the
// solve vector.
int compact_region_items(const fo::HostTables& t) {
  if (t.ce_ptr.empty()) return region_items(t);
  const int rows = t.cmax_half + fo::kCompactRing * fo::kStreamChunk;
  const int half = std::max(t.csm, t.n - t.csm);
  return std::max(rows, half);
}

size_t smem_bytes(const fo::HostTables& t, int lanes, int variant = FO_VARIANT_PIPELINED) {
  const int items = variant == FO_VARIANT_COMPACT ? compact_region_items(t) : region_items(t);
  return sizeof(double) * (32 + (size_t)items * lanes);
}

constexpr size_t kHeader = 256;  // queue counter at the start of the workspace
constexpr size_t kRoundsOffset = 64;  // the lockstep barrier words, inside the header
constexpr int kRoundsWords = 8;
constexpr int kMaxLanes = 256;

template <typename T>
size_t append(std::vector<char>& buf, const std::vector<T>& v) {
  size_t off = (buf.size() + 255) & ~size_t(255);
  buf.resize(off + v.size() * sizeof(T) + 1);
  if (!v.empty()) std::memcpy(buf.data() + off, v.data(), v.size() * sizeof(T));
  return off;
}

void fill_info(const fo::HostTables& t, fo_plan_info* info) {
  std::memset(info, 0, sizeof(*info));
  info->n = t.n;
  info->R = t.R;
  info->P = t.P;
  info->nnz_jac = t.nnz;
  info->ordering = t.ordering;
  info->nnz_lu = (int32_t)t.lu_col.size();
  info->nnz_l = t.nnz_l;
  info->nnz_u = t.nnz_u;
  info->lu_fma = t.lu_fma;
  info->solve_fma = t.solve_fma;
  info->jac_terms = (int32_t)t.jt_idx.size();
  info->stoich_nnz = (int32_t)t.s_rxn.size();
  info->scratch_doubles_per_cell = layout_of(t).items;
  info->smem_doubles_per_cell = region_items(t);
  info->compact_smem_doubles_per_cell = compact_region_items(t);
}

fo::SolveParams base_params(const fo_plan* plan) {
  fo::SolveParams p;
  std::memset(&p, 0, sizeof(p));
  p.t = plan->dev;
  p.sl = layout_of(plan->host);
  return p;
}

}  // namespace

extern "C" {

const char* fo_last_error(void) { return g_last_error.c_str(); }

int fo_analyze(const fo_mechanism_desc* mech, int32_t ordering, fo_plan_info* info, int32_t* perm) {
  if (!mech || !info) return fail(FO_E_INVALID, "null argument");
  try {
    fo::HostTables t;
    std::string err = fo::build_tables(*mech, ordering, &t);
    if (!err.empty()) return fail(FO_E_INVALID, err);
    fill_info(t, info);
    if (perm) std::memcpy(perm, t.perm.data(), sizeof(int32_t) * t.n);
  } catch (const std::bad_alloc&) {
    return fail(FO_E_ALLOC, "host allocation failed");
  }
  return FO_OK;
}

int fo_generate_check(const fo_mechanism_desc* mech, int32_t ordering, int32_t link, fo_gen_info* info) {
  if (!mech) return fail(FO_E_INVALID, "null argument");
  try {
    fo::HostTables t;
    std::string err = fo::build_tables(*mech, ordering, &t);
    if (!err.empty()) return fail(FO_E_INVALID, err);
    int rc = fo::gen_check(t, fo::GenOptions(), link != 0, info, &err);
    if (rc != FO_OK) return fail(rc, err);
  } catch (const std::bad_alloc&) {
    return fail(FO_E_ALLOC, "host allocation failed");
  }
  return FO_OK;
}

int fo_plan_create(const fo_mechanism_desc* mech, int32_t ordering, fo_plan** out) {
  if (!mech || !out) return fail(FO_E_INVALID, "null argument");
  *out = nullptr;
  fo_plan* plan = new (std::nothrow) fo_plan;
  if (!plan) return fail(FO_E_ALLOC, "host allocation failed");
  try {
    std::string err = fo::build_tables(*mech, ordering, &plan->host);
    if (!err.empty()) {
      delete plan;
      return fail(FO_E_INVALID, err);
    }
  } catch (const std::bad_alloc&) {
    delete plan;
    return fail(FO_E_ALLOC, "host allocation failed");
  }
  const fo::HostTables& t = plan->host;
  std::vector<char> buf;
  size_t o_perm = append(buf, t.perm), o_mass = append(buf, t.mass), o_react = append(buf, t.react),
         o_sptr = append(buf, t.s_ptr), o_srxn = append(buf, t.s_rxn), o_sval = append(buf, t.s_val),
         o_jrow = append(buf, t.j_row_ptr), o_jcol = append(buf, t.j_col), o_jsrc = append(buf, t.j_src),
         o_jtp = append(buf, t.jt_ptr), o_jti = append(buf, t.jt_idx), o_jtv = append(buf, t.jt_val),
         o_lur = append(buf, t.lu_row_ptr), o_lud = append(buf, t.lu_diag), o_luc = append(buf, t.lu_col),
         o_elp = append(buf, t.el_ptr), o_el = append(buf, t.el), o_sf = append(buf, t.sf),
         o_sb = append(buf, t.sb), o_jpos = append(buf, t.j_lu_pos), o_elpk = append(buf, t.elp),
         o_stp = append(buf, t.st_ptr), o_sts = append(buf, t.st_sp), o_stv = append(buf, t.st_val),
         o_css = append(buf, t.cs_split), o_csj = append(buf, t.cs_jsplit), o_cep_ptr = append(buf, t.ce_ptr),
         o_cep = append(buf, t.cep), o_cfa = append(buf, t.csf_a), o_cfb = append(buf, t.csf_b),
         o_cbb = append(buf, t.csb_b), o_cba = append(buf, t.csb_a);
  cudaError_t e = cudaGetDevice(&plan->device);
  if (e != cudaSuccess) {
    delete plan;
    return cuda_fail(e, "cudaGetDevice");
  }
  e = cudaMalloc(&plan->blob, buf.size());
  if (e != cudaSuccess) {
    delete plan;
    return cuda_fail(e, "cudaMalloc(plan tables)");
  }
  e = cudaMemcpy(plan->blob, buf.data(), buf.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(plan->blob);
    delete plan;
    return cuda_fail(e, "cudaMemcpy(plan tables)");
  }
  char* b = static_cast<char*>(plan->blob);
  fo::DevTables& d = plan->dev;
  d.n = t.n;
  d.R = t.R;
  d.P = t.P;
  d.nlu = (int)t.lu_col.size();
  d.nnzj = (int)t.j_col.size();
  d.perm = reinterpret_cast<const int32_t*>(b + o_perm);
  d.mass = reinterpret_cast<const double*>(b + o_mass);
  d.react = reinterpret_cast<const int32_t*>(b + o_react);
  d.s_ptr = reinterpret_cast<const int32_t*>(b + o_sptr);
  d.s_rxn = reinterpret_cast<const int32_t*>(b + o_srxn);
  d.s_val = reinterpret_cast<const double*>(b + o_sval);
  d.j_row_ptr = reinterpret_cast<const int32_t*>(b + o_jrow);
  d.j_col = reinterpret_cast<const int32_t*>(b + o_jcol);
  d.j_src = reinterpret_cast<const int32_t*>(b + o_jsrc);
  d.jt_ptr = reinterpret_cast<const int32_t*>(b + o_jtp);
  d.jt_idx = reinterpret_cast<const int32_t*>(b + o_jti);
  d.jt_val = reinterpret_cast<const double*>(b + o_jtv);
  d.lu_row_ptr = reinterpret_cast<const int32_t*>(b + o_lur);
  d.lu_diag = reinterpret_cast<const int32_t*>(b + o_lud);
  d.lu_col = reinterpret_cast<const int32_t*>(b + o_luc);
  d.el_ptr = reinterpret_cast<const int32_t*>(b + o_elp);
  d.el = reinterpret_cast<const int2*>(b + o_el);
  d.elp = t.elp.empty() ? nullptr : reinterpret_cast<const uint32_t*>(b + o_elpk);
  d.st_ptr = reinterpret_cast<const int32_t*>(b + o_stp);
  d.st_sp = reinterpret_cast<const int32_t*>(b + o_sts);
  d.st_val = reinterpret_cast<const double*>(b + o_stv);
  d.sf = reinterpret_cast<const int2*>(b + o_sf);
  d.sb = reinterpret_cast<const int2*>(b + o_sb);
  d.nsf = (int)(t.sf.size() / 2);
  d.nsb = (int)(t.sb.size() / 2);
  d.j_pos = reinterpret_cast<const int32_t*>(b + o_jpos);
  d.cs_split = reinterpret_cast<const int32_t*>(b + o_css);
  d.cs_jsplit = reinterpret_cast<const int32_t*>(b + o_csj);
  d.ce_ptr = reinterpret_cast<const int32_t*>(b + o_cep_ptr);
  d.cep = t.ce_ptr.empty() ? nullptr : reinterpret_cast<const uint32_t*>(b + o_cep);
  d.cmax_half = t.cmax_half;
  d.csm = t.csm;
  d.csf_a = reinterpret_cast<const int2*>(b + o_cfa);
  d.csf_b = reinterpret_cast<const int2*>(b + o_cfb);
  d.csb_b = reinterpret_cast<const int2*>(b + o_cbb);
  d.csb_a = reinterpret_cast<const int2*>(b + o_cba);
  d.ncsf_a = (int)(t.csf_a.size() / 2);
  d.ncsf_b = (int)(t.csf_b.size() / 2);
  d.ncsb_b = (int)(t.csb_b.size() / 2);
  d.ncsb_a = (int)(t.csb_a.size() / 2);
  d.max_row_len = t.max_row_len;
  d.region = region_items(t);
  d.has_constraints = 0;
  for (double m : t.mass)
    if (m == 0.0) d.has_constraints = 1;
  *out = plan;
  return FO_OK;
}

int fo_plan_info_get(const fo_plan* plan, fo_plan_info* info) {
  if (!plan || !info) return fail(FO_E_INVALID, "null argument");
  fill_info(plan->host, info);
  return FO_OK;
}

int fo_plan_destroy(fo_plan* plan) {
  if (!plan) return FO_OK;
  fo::gen_destroy(plan->gen);
  if (plan->blob) cudaFree(plan->blob);
  delete plan;
  return FO_OK;
}

int fo_plan_permutation(const fo_plan* plan, int32_t* perm) {
  if (!plan || !perm) return fail(FO_E_INVALID, "null argument");
  std::memcpy(perm, plan->host.perm.data(), sizeof(int32_t) * plan->host.n);
  return FO_OK;
}

int fo_plan_set_generation(fo_plan* plan, int32_t tile, int32_t solve_block) {
  if (!plan) return fail(FO_E_INVALID, "null plan");
  if (tile < 1 || tile > 16 || solve_block < 1 || solve_block > 64)
    return fail(FO_E_INVALID, "tile must be 1..16 and solve_block 1..64");
  std::lock_guard<std::mutex> lock(plan->gen_mutex);
  if (plan->gen && (plan->gen_options.tile != tile || plan->gen_options.solve_block != solve_block))
    return fail(FO_E_INVALID, "the plan's generated module was made with other options");
  plan->gen_options.tile = tile;
  plan->gen_options.solve_block = solve_block;
  return FO_OK;
}

int fo_plan_generate(fo_plan* plan, const char* cache_dir, fo_gen_info* info) {
  if (!plan) return fail(FO_E_INVALID, "null plan");
  std::lock_guard<std::mutex> lock(plan->gen_mutex);
  if (!plan->gen) {
    std::string err;
    fo_gen_info gi;
    int rc = fo::gen_create({&plan->host}, {plan->gen_options}, cache_dir, &plan->gen, &gi, &err);
    if (rc != FO_OK) return fail(rc, err);
    plan->gen_info = gi;
  }
  if (info) *info = plan->gen_info;
  return FO_OK;
}

int fo_workspace_bytes(const fo_plan* plan, int32_t slots, int32_t max_group_cells, size_t* bytes) {
  if (!plan || !bytes || slots <= 0 || max_group_cells <= 0) return fail(FO_E_INVALID, "bad argument");
  const int lanes = lanes_for(max_group_cells);
  *bytes = kHeader + sizeof(double) * (size_t)slots * (size_t)layout_of(plan->host).items * lanes;
  return FO_OK;
}

}  // extern "C"

namespace {

// Validate one batch and fill its kernel parameters (everything but the
// scratch and queue pointers).
int fill_params(const fo_plan* plan, const fo_options* opt, int32_t ngroups, const int32_t* group_offsets,
                int32_t max_group_cells, double* Y, int64_t ycs, int64_t yss, const double* k, int64_t kcs,
                int64_t krs, const double* atol, double rtol, double dt, double* memory, int64_t* counts,
                int32_t* status, fo::SolveParams* out, size_t* smem_out) {
  if (!plan || !opt || !group_offsets || !Y || !k || !atol || !memory || !counts || !status)
    return fail(FO_E_INVALID, "null argument");
  if (opt->tableau != FO_TABLEAU_ROS3 && opt->tableau != FO_TABLEAU_RODAS3)
    return fail(FO_E_INVALID, "unknown tableau");
  if (opt->variant != FO_VARIANT_PIPELINED && opt->variant != FO_VARIANT_PLAIN && opt->variant != FO_VARIANT_COMPACT &&
      opt->variant != FO_VARIANT_GENERATED)
    return fail(FO_E_INVALID, "unknown kernel variant");
  int variant = opt->variant;
  if (variant == FO_VARIANT_GENERATED && (max_group_cells <= 0 || max_group_cells > 32))
    return fail(FO_E_UNSUPPORTED, "FO_VARIANT_GENERATED runs groups of at most 32 cells");
  if (variant == FO_VARIANT_COMPACT && plan->dev.cep == nullptr) variant = FO_VARIANT_PIPELINED;
  if (variant == FO_VARIANT_PIPELINED && plan->dev.elp == nullptr) variant = FO_VARIANT_PLAIN;
  if (max_group_cells <= 0 || max_group_cells > kMaxLanes)
    return fail(FO_E_UNSUPPORTED, "group size must be 1..256 cells");
  if (!(dt > 0.0)) return fail(FO_E_INVALID, "dt must be positive");
  if (opt->max_steps < 0) return fail(FO_E_INVALID, "max_steps must be non-negative");
  const int lanes = lanes_for(max_group_cells);
  // the generated variant keeps nothing on chip but the reduction buffer,
  // plus the projection's dense work row for a constrained mechanism
  const size_t smem = variant == FO_VARIANT_GENERATED
                          ? sizeof(double) * (32 + (plan->dev.has_constraints ? (size_t)plan->host.n * lanes : 0))
                          : smem_bytes(plan->host, lanes, variant);
  int dev = 0, smem_max = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  if (smem > (size_t)smem_max)
    return fail(FO_E_UNSUPPORTED, "species x group size exceed shared memory: use smaller groups");
  fo::SolveParams p = base_params(plan);
  p.o.tab = kTableaus[opt->tableau];
  p.o.controller = opt->controller;
  p.o.b = opt->b;
  p.o.safety = opt->safety;
  p.o.fac_min = opt->fac_min;
  p.o.fac_max = opt->fac_max;
  p.o.carry = opt->carry;
  p.o.quantize = opt->quantize;
  p.o.carry_memory = opt->carry_memory;
  p.o.max_steps = opt->max_steps;
  p.o.variant = variant;
  if (opt->loop != FO_LOOP_ALGORITHM && opt->loop != FO_LOOP_RESTARTING && opt->loop != FO_LOOP_BACKWARD_EULER)
    return fail(FO_E_INVALID, "unknown loop");
  p.o.loop = opt->loop;
  p.o.step_change_rows = opt->step_change_rows;
  if (opt->loop == FO_LOOP_BACKWARD_EULER) {
    if (opt->nreductions < 0 || opt->nreductions > 8) return fail(FO_E_INVALID, "nreductions must be 0..8");
    for (int i = 0; i < opt->nreductions; ++i)
      if (!(opt->reductions[i] > 0.0) || !std::isfinite(opt->reductions[i]))
        return fail(FO_E_INVALID, "backward Euler reductions must be positive and finite");
    if (!std::isfinite(opt->small)) return fail(FO_E_INVALID, "small must be finite");
    p.o.max_iterations = opt->max_iterations;
    p.o.nreductions = opt->nreductions;
    for (int i = 0; i < 8; ++i) p.o.reductions[i] = i < opt->nreductions ? opt->reductions[i] : 1.0;
    p.o.small = opt->small;
  }
  // the pipelined kernel needs the packed stream (positions below 65,536 and
  // rows shorter than 32,767 entries); larger mechanisms run the plain loops
  p.o.k_exp = 3.0;  // embedded order 2 for both tableaus
  p.ngroups = ngroups;
  p.group_offsets = group_offsets;
  p.Y = Y;
  p.ycs = ycs;
  p.yss = yss;
  p.k = k;
  p.kcs = kcs;
  p.krs = krs;
  p.atol = atol;
  p.rtol = rtol;
  p.dt = dt;
  p.memory = memory;
  p.counts = reinterpret_cast<long long*>(counts);
  p.status = status;
  p.lanes = lanes;
  p.slot_doubles = p.sl.items * lanes;
  *out = p;
  *smem_out = smem;
  return FO_OK;
}

}  // namespace

struct fo_multi {
  int nb = 0, grid = 0, lanes = 0;
  size_t smem = 0;
  fo::GenModule* gen = nullptr;          // the generated module of every batch's mechanism
  fo::SolveParams* d_batches = nullptr;  // in the workspace
  int32_t* d_starts = nullptr;
  int32_t* d_queue = nullptr;
  double* d_scratch = nullptr;
  int64_t slot_doubles = 0;
  unsigned int* d_rounds = nullptr;      // lockstep rounds' barrier words, or null
};

namespace {

struct MultiLayout {
  int lanes = 0, total = 0, grid = 0;
  int64_t items = 0;
  size_t params_off = 0, starts_off = 0, scratch_off = 0, bytes = 0;
};

int multi_layout(int32_t nb, const fo_batch_desc* b, int32_t slots, MultiLayout* L) {
  if (nb <= 0 || !b) return fail(FO_E_INVALID, "no batches");
  for (int i = 0; i < nb; ++i) {
    if (!b[i].plan) return fail(FO_E_INVALID, "null plan");
    if (b[i].ngroups < 0) return fail(FO_E_INVALID, "negative group count");
    if (b[i].max_group_cells <= 0 || b[i].max_group_cells > kMaxLanes)
      return fail(FO_E_UNSUPPORTED, "group size must be 1..256 cells");
    L->lanes = std::max(L->lanes, lanes_for(b[i].max_group_cells));
    L->items = std::max<int64_t>(L->items, layout_of(b[i].plan->host).items);
    L->total += b[i].ngroups;
  }
  L->grid = slots > 0 ? std::min(slots, std::max(L->total, 1)) : std::max(L->total, 1);
  L->params_off = kHeader;
  L->starts_off = (L->params_off + sizeof(fo::SolveParams) * nb + 255) & ~size_t(255);
  L->scratch_off = (L->starts_off + sizeof(int32_t) * (nb + 1) + 255) & ~size_t(255);
  L->bytes = L->scratch_off + sizeof(double) * (size_t)L->grid * (size_t)L->items * L->lanes;
  return FO_OK;
}

}  // namespace

extern "C" {

int fo_solve(const fo_plan* plan, const fo_options* opt, int32_t ngroups, const int32_t* group_offsets,
             int32_t max_group_cells, double* Y, int64_t y_cell_stride, int64_t y_species_stride, const double* k,
             int64_t k_cell_stride, int64_t k_reaction_stride, const double* atol, double rtol, double dt,
             double* memory, int64_t* counts, int32_t* status, void* workspace, size_t workspace_bytes,
             int32_t slots, double* trace, int32_t trace_cap, int32_t* trace_len, void* stream) {
  if (!workspace) return fail(FO_E_INVALID, "null workspace");
  if (ngroups <= 0) return FO_OK;
  if (opt && opt->variant == FO_VARIANT_GENERATED && plan && !plan->gen)
    return fail(FO_E_UNSUPPORTED, "FO_VARIANT_GENERATED needs fo_plan_generate on this plan first");
  fo::SolveParams p;
  size_t smem = 0;
  int rc = fill_params(plan, opt, ngroups, group_offsets, max_group_cells, Y, y_cell_stride, y_species_stride, k,
                       k_cell_stride, k_reaction_stride, atol, rtol, dt, memory, counts, status, &p, &smem);
  if (rc != FO_OK) return rc;
  const int grid = slots > 0 ? (slots < ngroups ? slots : ngroups) : ngroups;
  size_t need = 0;
  fo_workspace_bytes(plan, grid, max_group_cells, &need);
  if (workspace_bytes < need) return fail(FO_E_WORKSPACE, "workspace too small");
  p.scratch = reinterpret_cast<double*>(static_cast<char*>(workspace) + kHeader);
  p.trace = trace;
  p.trace_cap = trace ? trace_cap : 0;
  p.trace_len = trace_len;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (slots > 0) {
    p.queue = static_cast<int32_t*>(workspace);
    e = cudaMemsetAsync(workspace, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(queue)");
  } else {
    p.queue = nullptr;
  }
  // lockstep rounds (fo_options.lockstep): barrier words in the workspace
  // header, zeroed for every launch
  p.rounds = nullptr;
  p.round_attempts = 1;
  if (opt->lockstep && p.o.variant == FO_VARIANT_GENERATED && p.o.loop == FO_LOOP_ALGORITHM) {
    p.rounds = reinterpret_cast<unsigned int*>(static_cast<char*>(workspace) + kRoundsOffset);
    e = cudaMemsetAsync(p.rounds, 0, kRoundsWords * sizeof(unsigned int), s);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(rounds)");
  }
  if (p.o.variant == FO_VARIANT_GENERATED) e = fo::gen_launch(plan->gen, p, grid, smem, s);
  else e = fo::launch_solve(p, grid, smem, s);
  if (e != cudaSuccess) return cuda_fail(e, "solve kernel launch");
  return FO_OK;
}

int fo_multi_workspace_bytes(int32_t nbatches, const fo_batch_desc* batches, int32_t slots, size_t* bytes) {
  if (!bytes) return fail(FO_E_INVALID, "null argument");
  MultiLayout L;
  int rc = multi_layout(nbatches, batches, slots, &L);
  if (rc != FO_OK) return rc;
  *bytes = L.bytes;
  return FO_OK;
}

int fo_multi_prepare(int32_t nb, const fo_batch_desc* b, void* workspace, size_t workspace_bytes, int32_t slots,
                     fo_multi** out) {
  if (!out || !workspace) return fail(FO_E_INVALID, "null argument");
  *out = nullptr;
  MultiLayout L;
  int rc = multi_layout(nb, b, slots, &L);
  if (rc != FO_OK) return rc;
  if (workspace_bytes < L.bytes) return fail(FO_E_WORKSPACE, "workspace too small");
  // largest mechanisms first, so the queue's tail holds the cheapest groups
  std::vector<int> order(nb);
  for (int i = 0; i < nb; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return layout_of(b[x].plan->host).items > layout_of(b[y].plan->host).items;
  });
  std::vector<fo::SolveParams> params(nb);
  std::vector<int32_t> starts(nb + 1, 0);
  size_t smem = 0;
  for (int j = 0; j < nb; ++j) {
    const fo_batch_desc& d = b[order[j]];
    size_t sm = 0;
    rc = fill_params(d.plan, &d.opt, d.ngroups, d.group_offsets, d.max_group_cells, d.Y, d.y_cell_stride,
                     d.y_species_stride, d.k, d.k_cell_stride, d.k_reaction_stride, d.atol, d.rtol, d.dt, d.memory,
                     d.counts, d.status, &params[j], &sm);
    if (rc != FO_OK) return rc;
    smem = std::max(smem, params[j].o.variant == FO_VARIANT_GENERATED ? sm
                                                                       : smem_bytes(d.plan->host, L.lanes,
                                                                                    params[j].o.variant));
    starts[j + 1] = starts[j] + d.ngroups;
  }
  // the generated variant: one module with every distinct mechanism, each
  // batch pointing at its own by index (all batches generated, or none)
  int ngen = 0;
  for (const auto& p : params) ngen += p.o.variant == FO_VARIANT_GENERATED ? 1 : 0;
  if (ngen != 0 && ngen != nb)
    return fail(FO_E_UNSUPPORTED, "one launch runs either the generated variant for every batch or for none");
  std::vector<const fo::HostTables*> tables;
  std::vector<fo::GenOptions> gen_opts;
  if (ngen) {
    if (L.lanes != 32) return fail(FO_E_UNSUPPORTED, "FO_VARIANT_GENERATED runs groups of at most 32 cells");
    for (int j = 0; j < nb; ++j) {
      const fo_plan* pl = b[order[j]].plan;
      auto it = std::find(tables.begin(), tables.end(), &pl->host);
      params[j].o.gen_index = (int)(it - tables.begin());
      if (it == tables.end()) {
        tables.push_back(&pl->host);
        gen_opts.push_back(pl->gen_options);
      }
    }
  }
  int dev = 0, smem_max = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  if (smem > (size_t)smem_max) return fail(FO_E_UNSUPPORTED, "species x group size exceed shared memory");
  char* ws = static_cast<char*>(workspace);
  fo_multi* m = new (std::nothrow) fo_multi;
  if (!m) return fail(FO_E_ALLOC, "host allocation failed");
  if (ngen) {
    std::string err;
    rc = fo::gen_create(tables, gen_opts, nullptr, &m->gen, nullptr, &err);
    if (rc != FO_OK) {
      delete m;
      return fail(rc, err);
    }
  }
  m->nb = nb;
  m->grid = L.grid;
  m->lanes = L.lanes;
  m->smem = smem;
  m->d_batches = reinterpret_cast<fo::SolveParams*>(ws + L.params_off);
  m->d_starts = reinterpret_cast<int32_t*>(ws + L.starts_off);
  m->d_queue = reinterpret_cast<int32_t*>(ws);
  m->d_scratch = reinterpret_cast<double*>(ws + L.scratch_off);
  m->slot_doubles = L.items * L.lanes;
  // lockstep rounds when every batch asks for them and runs the generated
  // Algorithm loop, and every slot is resident;
  // each batch makes as many attempts per round as the largest mechanism's
  // attempt costs over its own (LU and three solves), at least one
  bool lockstep = ngen == nb;
  int64_t cost_max = 1;
  for (int j = 0; j < nb; ++j) {
    const fo_batch_desc& d = b[order[j]];
    lockstep = lockstep && d.opt.lockstep && params[j].o.loop == FO_LOOP_ALGORITHM;
    cost_max = std::max<int64_t>(cost_max, d.plan->host.lu_fma + 3 * d.plan->host.solve_fma);
  }
  if (lockstep) lockstep = fo::gen_resident(m->gen, true, m->grid, smem);
  m->d_rounds = lockstep ? reinterpret_cast<unsigned int*>(ws + kRoundsOffset) : nullptr;
  for (int j = 0; j < nb; ++j) {
    fo::SolveParams& p = params[j];
    p.scratch = m->d_scratch;
    p.slot_doubles = m->slot_doubles;
    p.lanes = L.lanes;
    p.queue = m->d_queue;
    p.rounds = m->d_rounds;
    const int64_t cost = std::max<int64_t>(1, b[order[j]].plan->host.lu_fma + 3 * b[order[j]].plan->host.solve_fma);
    p.round_attempts = (int)std::max<int64_t>(1, (cost_max + cost / 2) / cost);
  }
  e = cudaMemcpy(m->d_batches, params.data(), sizeof(fo::SolveParams) * nb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(m->d_starts, starts.data(), sizeof(int32_t) * (nb + 1), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    fo::gen_destroy(m->gen);
    delete m;
    return cuda_fail(e, "cudaMemcpy(batch table)");
  }
  *out = m;
  return FO_OK;
}

int fo_multi_launch(const fo_multi* m, void* stream) {
  if (!m) return fail(FO_E_INVALID, "null argument");
  if (m->d_rounds) {
    cudaError_t z = cudaMemsetAsync(m->d_rounds, 0, kRoundsWords * sizeof(unsigned int),
                                    static_cast<cudaStream_t>(stream));
    if (z != cudaSuccess) return cuda_fail(z, "cudaMemsetAsync(rounds)");
  }
  cudaError_t e = m->gen ? fo::gen_launch_multi(m->gen, m->d_batches, m->nb, m->d_starts, m->d_queue,
                                                m->d_scratch, m->slot_doubles, m->grid, m->smem,
                                                m->d_rounds != nullptr, static_cast<cudaStream_t>(stream))
                         : fo::launch_solve_multi(m->d_batches, m->nb, m->d_starts, m->d_queue, m->d_scratch,
                                                  m->slot_doubles, m->grid, m->lanes, m->smem,
                                                  static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "multi solve launch");
  return FO_OK;
}

int fo_multi_destroy(fo_multi* m) {
  if (m) fo::gen_destroy(m->gen);
  delete m;
  return FO_OK;
}

}  // extern "C"

namespace {

fo::AdjLayout adjoint_layout(const fo::HostTables& t, int max_steps) {
  fo::AdjLayout a;
  int64_t o = layout_of(t).items;
  a.ys = o; o += (int64_t)max_steps * t.n;
  a.u = o; o += 4LL * t.n;
  a.kbar = o; o += 4LL * t.n;
  a.fbar = o; o += 4LL * t.n;
  a.ybar = o; o += t.n;
  a.g = o; o += t.n;
  a.jbar = o; o += (int64_t)t.j_col.size();
  a.dbar = o; o += (int64_t)t.R * t.P;
  bool constrained = false;
  for (double m : t.mass) constrained = constrained || m == 0.0;
  a.yp = o; o += constrained ? (int64_t)fo::kMaxProjectionUpdates * t.n : 0;
  a.pdelta = o; o += constrained ? t.n : 0;
  a.pmu = o; o += constrained ? t.n : 0;
  a.items = o;
  return a;
}

}  // namespace

extern "C" {

int fo_adjoint_workspace_bytes(const fo_plan* plan, int32_t ngroups, int32_t max_group_cells, int32_t max_steps,
                               size_t* bytes) {
  if (!plan || !bytes || ngroups <= 0 || max_group_cells <= 0 || max_steps < 0)
    return fail(FO_E_INVALID, "bad argument");
  *bytes = kHeader + sizeof(double) * (size_t)ngroups * (size_t)adjoint_layout(plan->host, max_steps).items *
                         lanes_for(max_group_cells);
  return FO_OK;
}

int fo_adjoint_interval(const fo_plan* plan, const fo_options* opt, int32_t ngroups, const int32_t* group_offsets,
                        int32_t max_group_cells, const double* Y, int64_t ycs, int64_t yss, const double* k,
                        int64_t kcs, int64_t krs, const double* atol, double dt, const int32_t* step_ptr,
                        const double* steps, int32_t max_steps, const int32_t* proj_ptr, const double* proj_steps,
                        int32_t mode, double* lam, int64_t lcs, int64_t lss,
                        double* thbar, int64_t tcs, int64_t trs, double* Yout, int64_t ocs, int64_t oss,
                        int32_t* status, void* workspace, size_t workspace_bytes, void* stream) {
  if (ngroups <= 0) return FO_OK;
  if (!Y || !step_ptr || !steps || !status || !workspace) return fail(FO_E_INVALID, "null argument");
  if (mode != 0 && mode != 1) return fail(FO_E_INVALID, "mode must be 0 (replay) or 1 (adjoint)");
  if (mode == 0 && !Yout) return fail(FO_E_INVALID, "replay needs Yout");
  if (mode == 1 && (!lam || !thbar)) return fail(FO_E_INVALID, "adjoint needs lam and thbar");
  if (opt && opt->loop == FO_LOOP_BACKWARD_EULER)
    return fail(FO_E_UNSUPPORTED, "the adjoint replays Rosenbrock steps: backward Euler has none");
  fo::AdjParams a;
  std::memset(&a, 0, sizeof(a));
  size_t smem = 0;
  // the group memory/counters/status of fill_params are not used by the adjoint
  int rc = fill_params(plan, opt, ngroups, group_offsets, max_group_cells, const_cast<double*>(Y), ycs, yss, k, kcs,
                       krs, atol, 0.0, dt, reinterpret_cast<double*>(workspace), reinterpret_cast<int64_t*>(workspace),
                       status, &a.p, &smem);
  if (rc != FO_OK) return rc;
  size_t need = 0;
  fo_adjoint_workspace_bytes(plan, ngroups, max_group_cells, max_steps, &need);
  if (workspace_bytes < need) return fail(FO_E_WORKSPACE, "workspace too small");
  a.al = adjoint_layout(plan->host, max_steps);
  const bool generated = a.p.o.variant == FO_VARIANT_GENERATED && plan->gen != nullptr;
  if (generated) {
    // the generated adjoint keeps nothing else on chip but the projection's
    // dense work row (constrained mechanisms)
    smem = sizeof(double) * (32 + (plan->dev.has_constraints ? (size_t)plan->host.n * a.p.lanes : 0));
  } else if (a.p.o.variant == FO_VARIANT_COMPACT || a.p.o.variant == FO_VARIANT_GENERATED) {
    // the table-driven transposed solves need the whole vector on chip
    a.p.o.variant = plan->dev.elp ? FO_VARIANT_PIPELINED : FO_VARIANT_PLAIN;
    smem = smem_bytes(plan->host, a.p.lanes, a.p.o.variant);
  }
  a.p.slot_doubles = a.al.items * a.p.lanes;
  a.p.scratch = reinterpret_cast<double*>(static_cast<char*>(workspace) + kHeader);
  a.Ycp = Y;
  a.ycs = ycs;
  a.yss = yss;
  a.lam = lam;
  a.lcs = lcs;
  a.lss = lss;
  a.thbar = thbar;
  a.tcs = tcs;
  a.trs = trs;
  a.Yout = Yout;
  a.ocs = ocs;
  a.oss = oss;
  a.step_ptr = step_ptr;
  a.steps = steps;
  if ((proj_ptr == nullptr) != (proj_steps == nullptr))
    return fail(FO_E_INVALID, "proj_ptr and proj_steps go together");
  if (proj_ptr && !plan->dev.has_constraints)
    return fail(FO_E_INVALID, "projection updates given for a mechanism without algebraic species");
  a.proj_ptr = proj_ptr;
  a.proj_steps = proj_steps;
  a.max_steps = max_steps;
  a.mode = mode;
  a.status = status;
  cudaError_t e = generated ? fo::gen_launch_adjoint(plan->gen, a, ngroups, smem, static_cast<cudaStream_t>(stream))
                            : fo::launch_adjoint(a, ngroups, a.p.lanes, smem, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "adjoint kernel launch");
  return FO_OK;
}

static int eval_common(const fo_plan* plan, int32_t C, const double* Y, int64_t ycs, int64_t yss, const double* k,
                       int64_t kcs, int64_t krs, double* out, int want_jac, void* stream) {
  if (!plan || !Y || !k || !out) return fail(FO_E_INVALID, "null argument");
  if (C <= 0) return FO_OK;
  fo::SolveParams p = base_params(plan);
  p.Y = const_cast<double*>(Y);
  p.ycs = ycs;
  p.yss = yss;
  p.k = k;
  p.kcs = kcs;
  p.krs = krs;
  p.lanes = 64;
  p.slot_doubles = p.sl.items * p.lanes;
  const int blocks = (C + p.lanes - 1) / p.lanes;
  void* scratch = nullptr;
  cudaError_t e = cudaMalloc(&scratch, sizeof(double) * (size_t)blocks * p.slot_doubles);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(eval scratch)");
  p.scratch = static_cast<double*>(scratch);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  e = fo::launch_eval(p, C, want_jac, out, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(scratch);
  if (e != cudaSuccess) return cuda_fail(e, "eval kernel");
  return FO_OK;
}

int fo_eval_rhs(const fo_plan* plan, int32_t C, const double* Y, int64_t ycs, int64_t yss, const double* k,
                int64_t kcs, int64_t krs, double* F, void* stream) {
  return eval_common(plan, C, Y, ycs, yss, k, kcs, krs, F, 0, stream);
}

int fo_eval_jac(const fo_plan* plan, int32_t C, const double* Y, int64_t ycs, int64_t yss, const double* k,
                int64_t kcs, int64_t krs, double* J, void* stream) {
  return eval_common(plan, C, Y, ycs, yss, k, kcs, krs, J, 1, stream);
}

}  // extern "C"
