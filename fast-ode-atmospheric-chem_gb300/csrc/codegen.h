// Per-mechanism code generation: the factorization of alpha*M - J and the two
// triangular solves of one mechanism as straight-line PTX, every operand at an
// immediate offset from a lane's base pointer. The integrator kernel compiled
// as relocatable device code (generated.cu) calls them; jit.cpp links the
// two into one module per mechanism.
#pragma once

#include <cstdint>
#include <string>

#include "symbolic.h"

namespace fo {

struct GenOptions {
  // rows (and columns) of the register tiles of the factorization
  int tile = 6;
  // rows of a block of the triangular solves
  int solve_block = 8;
};

// PTX (ISA 9.0, sm_103a) defining
//   .visible .func fo_gen_factor(.param .b64 lu, .param .b64 negj, .param .f64 alpha)
//   .visible .func fo_gen_solve(.param .b64 lu, .param .b64 x)
// for a group of 32 lanes: lu, negj and x point at this lane's item 0 of a
// per-lane array laid out item-major with 32 lanes (item q at byte offset
// 256 q). fo_gen_factor assembles alpha*M - J from the negated Jacobian values
// (assembly order) and factors it in place in the LU storage order of `t`,
// with the same operations, in the same order per entry, as the row-by-row
// elimination (every entry receives its updates fma(-l, u, a) in ascending
// pivot order; multipliers a * (1 / pivot); the diagonal keeps 1 / pivot).
// fo_gen_solve overwrites x with (LU)^-1 x: forward then backward
// substitution, each row's sum in ascending column order.
std::string generate_ptx(const HostTables& t, const GenOptions& o, int64_t* fma_count = nullptr);

}  // namespace fo
