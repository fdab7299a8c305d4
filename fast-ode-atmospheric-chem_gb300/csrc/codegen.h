// Per-mechanism code generation: the factorization of alpha*M - J and the two
// triangular solves of one mechanism as straight-line PTX, every operand at an
// immediate offset from a lane's base pointer. The integrator kernel compiled
// as relocatable device code (generated.cu) calls them; jit.cpp links the
// two into one module per mechanism.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "symbolic.h"

namespace fo {

struct GenOptions {
  // rows (and columns) of the register tiles of the factorization
  int tile = 6;
  // rows of a block of the triangular solves
  int solve_block = 8;
  // values of later blocks the backward solve keeps in registers per block
  int solve_keep = 16;
  // instructions per separately compiled piece of the factorization (whole
  // row blocks; a block longer than this is a piece of its own)
  int piece_lines = 40000;
};

// PTX (ISA 9.0, sm_103a) defining
//   .visible .func fo_gen_factor(.param .b64 base, .param .b64 alpha, .param .b32 mech)
//   .visible .func fo_gen_solve(.param .b64 base, .param .b32 mech)
// for a group of 32 lanes: base points at this lane's item 0 of its scratch
// slot, laid out item-major with 32 lanes (item q at byte offset 256 q); the
// LU storage, the Jacobian values and the solve vector sit at the item
// offsets of the plan's scratch layout (layout.h). fo_gen_factor assembles
// alpha*M - J from the negated Jacobian values (assembly order) and factors
// it in place in the LU storage order of `t`, with the same operations, in
// the same order per entry, as the row-by-row elimination (every entry
// receives its updates fma(-l, u, a) in ascending pivot order; multipliers
// a * (1 / pivot); the diagonal keeps 1 / pivot). fo_gen_solve overwrites the
// solve vector with (LU)^-1 of it: forward then backward substitution, each
// row's sum in ascending column order. A third function,
//   .visible .func fo_gen_solve_t(.param .b64 base, .param .b32 mech)
// overwrites the solve vector with (LU)^-T of it for the adjoint, with the
// operations and order of its table-driven transposed solve. `mech` is
// ignored (one mechanism).
std::string generate_ptx(const HostTables& t, const GenOptions& o, int64_t* fma_count = nullptr);

// The same for several mechanisms in one module: `mech` is the mechanism's
// index in `ts` and selects its code.
std::string generate_ptx(const std::vector<const HostTables*>& ts, const std::vector<GenOptions>& os,
                         int64_t* fma_count = nullptr);

}  // namespace fo
