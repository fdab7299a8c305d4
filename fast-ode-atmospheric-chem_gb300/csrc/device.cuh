// Device-side data structures shared by the kernels of the integrator.
#pragma once

#include <vector_types.h>

#include <cstdint>

#include "stream.h"

namespace fo {

// Index tables of one plan (device pointers), in the permuted numbering.
struct DevTables {
  int n, R, P, nlu, nnzj;
  const int32_t* perm;        // n: original species of permuted index p
  const double* mass;         // n (permuted)
  const int32_t* react;       // R*P permuted species, n = a factor of one
  const int32_t* s_ptr;       // n+1
  const int32_t* s_rxn;
  const double* s_val;
  const int32_t* st_ptr;      // R+1: S by reactions
  const int32_t* st_sp;       // permuted species
  const double* st_val;
  const int32_t* j_row_ptr;   // n+1
  const int32_t* j_col;       // nnzj
  const int32_t* j_src;       // nnzj original pattern entry
  const int32_t* jt_ptr;      // nnzj+1
  const int32_t* jt_idx;      // j*P+p
  const double* jt_val;       // -S[i,j]
  const int32_t* lu_row_ptr;  // n+1
  const int32_t* lu_diag;     // n
  const int32_t* lu_col;      // nlu
  const int32_t* el_ptr;      // n+1: elimination stream rows (entries)
  const int2* el;             // stream entries (x, y)
  const uint32_t* elp;        // the stream packed to 32 bits, or null
  const int2* sf;             // forward-solve stream
  const int2* sb;             // backward-solve stream
  int nsf, nsb;               // entries of each solve stream
  const int32_t* j_pos;       // nnzj: position of each Jacobian entry in the LU storage
  // the compact variant (null cep when the tables do not fit)
  const int32_t* cs_split;    // n: first slot of each row's second pass
  const int32_t* cs_jsplit;   // n: first Jacobian entry of each row's second pass
  const int32_t* ce_ptr;      // 2n+1: the passes' entries
  const uint32_t* cep;        // the passes' entries, packed
  int cmax_half;              // slots of the largest pass
  int csm;                    // rows of the solve vector's first half
  const int2* csf_a;          // the split solves' streams
  const int2* csf_b;
  const int2* csb_b;
  const int2* csb_a;
  int ncsf_a, ncsf_b, ncsb_b, ncsb_a;
  int max_row_len;            // longest row of the filled pattern
  int region;                 // shared-memory items per lane (work row / ring / solve vector)
  int has_constraints;
};

struct DevTableau {
  double gamma;
  int S;
  double a[4][4], c[4][4], m[4], e[4];
  int new_forcing[4];
};

struct DevOptions {
  DevTableau tab;
  int controller;  // 0 h211b, 1 elementary
  double b, safety, fac_min, fac_max;
  int carry, quantize, carry_memory, max_steps;
  int variant;     // FO_VARIANT_*
  int gen_index;   // FO_VARIANT_GENERATED: the mechanism's index in its generated module
  int loop;        // FO_LOOP_*
  int step_change_rows;
  double k_exp;    // embedded order + 1
  // backward Euler (FO_LOOP_BACKWARD_EULER)
  int max_iterations, nreductions;
  double reductions[8];
  double small;
};

// Per-lane scratch layout, in items (each item is `lanes` doubles).
struct ScratchLayout {
  int64_t lu, negj, d, r, y, ynew, f0, ft, yr, k;  // offsets
  int64_t xs;                                      // the generated solves' vector (n items)
  int64_t items;                                   // total items per lane
};

struct SolveParams {
  DevTables t;
  DevOptions o;
  ScratchLayout sl;
  int ngroups;
  const int32_t* group_offsets;  // device, ngroups+1
  double* Y;
  int64_t ycs, yss;
  const double* k;
  int64_t kcs, krs;
  const double* atol;            // original order
  double rtol, dt;
  double* memory;
  long long* counts;
  int32_t* status;
  double* scratch;               // per slot: items * lanes doubles
  int64_t slot_doubles;
  int32_t* queue;                // work counter (persistent mode) or null
  int lanes;                     // threads per block (multiple of 32)
  double* trace;
  int trace_cap;
  int32_t* trace_len;
  unsigned int* rounds;          // lockstep rounds (five barrier words), or null
  int round_attempts;            // attempts per round
};

// Extra per-lane scratch of the adjoint (items after the forward layout).
struct AdjLayout {
  int64_t ys;     // max_steps * n: state at the start of every step
  int64_t u;      // 4n: stage points of the stages that evaluate F anew
  int64_t kbar;   // 4n
  int64_t fbar;   // 4n
  int64_t ybar;   // n
  int64_t g;      // n: a forcing vector-Jacobian product
  int64_t jbar;   // nnzj
  int64_t dbar;   // R*P
  int64_t yp;     // constrained systems: kMaxProjectionUpdates * n, the state before each projection update
  int64_t pdelta; // n: a projection update's Newton correction
  int64_t pmu;    // n: its adjoint
  int64_t items;  // total items per lane, forward layout included
};

// The projection's update limit (fastode/solvers.py:100-178: ten updates and
// the check after them), the most updates one call can apply.
constexpr int kMaxProjectionUpdates = 11;

struct AdjParams {
  SolveParams p;        // tables, tableau, forward scratch layout, rate constants, group offsets, dt
  AdjLayout al;
  const double* Ycp;    // state at the interval start (checkpoint)
  int64_t ycs, yss;
  double* lam;          // in: dL/dY at the interval end; out: dL/dY at the interval start
  int64_t lcs, lss;
  double* thbar;        // accumulated dL/dlog k per cell
  int64_t tcs, trs;
  double* Yout;         // replay mode: the interval's end state
  int64_t ocs, oss;
  const int32_t* step_ptr;  // ngroups+1
  const double* steps;      // accepted step sizes of the interval
  int max_steps;
  const int32_t* proj_ptr;  // ngroups+1, or null: the projection updates of each group
  const double* proj_steps; // their accepted line-search steps
  int mode;             // 0 replay, 1 adjoint
  int32_t* status;
};

}  // namespace fo
