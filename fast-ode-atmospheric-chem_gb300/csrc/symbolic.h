// Host-side symbolic analysis of a mass-action mechanism: fill-reducing
// ordering, pivot-free sparse LU structure and the index tables the device
// integrator walks. No CUDA here; the plan's tables are uploaded by abi.cu.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "fastode_gb300.h"
#include "stream.h"

namespace fo {


// Everything the device needs, in the permuted species numbering
// (p = 0..n-1 is the p-th eliminated species, perm[p] its original index).
struct HostTables {
  int n = 0, R = 0, P = 0, nnz = 0;
  int ordering = 0;
  std::vector<int32_t> perm, iperm;
  std::vector<double> mass;            // permuted

  // rates: react_p[j*P+p] = permuted species or n (a factor of one)
  std::vector<int32_t> react;
  // stoichiometry rows in permuted order: (reaction, coefficient)
  std::vector<int32_t> s_ptr, s_rxn;
  std::vector<double> s_val;
  // the same by reactions (columns of S): (permuted species, coefficient)
  std::vector<int32_t> st_ptr, st_sp;
  std::vector<double> st_val;

  // Jacobian values in assembly order (permuted row-major):
  // entry q sits in permuted row r with j_row_ptr[r] <= q < j_row_ptr[r+1],
  // permuted column j_col[q], original pattern entry j_src[q]
  std::vector<int32_t> j_row_ptr, j_col, j_src;
  // value map of entry q: terms jt_ptr[q]..jt_ptr[q+1], jp index and -S[i,j]
  std::vector<int32_t> jt_ptr, jt_idx;
  std::vector<double> jt_val;

  // LU storage: row r holds L entries (columns < r, ascending), the diagonal,
  // then U entries (columns > r, ascending)
  std::vector<int32_t> lu_row_ptr, lu_diag, lu_col;
  // position of the Jacobian entry q inside the LU storage
  std::vector<int32_t> j_lu_pos;

  // Elimination stream: for row r, entries el[2*t], el[2*t+1] for
  // el_ptr[r] <= t < el_ptr[r+1], padded to a multiple of kStreamChunk.
  //   update  (x >= 0):          w[y] -= l * lu[x]    (x: a U entry of an earlier row)
  //   marker  (x < 0, y >= 0):   l = w[y] * lu[-1-x]  (-1-x = diagonal slot of row k, which
  //                              holds 1/pivot); l is stored in the next L slot of row r
  //   no-op   (x = -1, y = -1):  padding
  // y is a slot of row r's own pattern: w[y] stands for lu[lu_row_ptr[r] + y].
  std::vector<int32_t> el_ptr, el;
  int max_row_len = 0;
  // The same stream packed to 32 bits per entry, (position << 16) | slot,
  // slot bit 15 set for a multiplier, slot 0x7fff for padding; empty when a
  // position or a slot does not fit (the plain kernel then runs instead).
  std::vector<uint32_t> elp;

  // Compact factorization and solves (FO_VARIANT_COMPACT), which keep half a
  // row and half the solve vector in shared memory. Row r is eliminated in two
  // passes over its slots, A = [0, cs_split[r]) and B = [cs_split[r], len):
  // A is the elimination restricted to the row's leading columns (its
  // multipliers are stored in the LU storage as they are made); B applies
  // every multiplier's updates of the trailing columns in the same order,
  // reloading the multipliers A made, and makes the rest. ce_ptr[2r + pass]
  // delimits the pass's entries in cep, packed as elp with slots relative to
  // the pass and kReloadSlot marking a reload (l = lu[position]); padded to
  // whole chunks. cs_jsplit[r] is the first Jacobian entry (assembly order)
  // of pass B. Empty when a slot or a position does not fit.
  std::vector<int32_t> cs_split, cs_jsplit, ce_ptr;
  std::vector<uint32_t> cep;
  int cmax_half = 0;
  // The split solves: rows [0, csm) and [csm, n) are the two halves of the
  // vector. Four streams like sf/sb, one per phase (forward over the first
  // half, forward over the second, backward over the second, backward over
  // the first): an entry's operand is the staged half in shared memory
  // (column relative to the half) or, with kGlobalOperand set, the finished
  // other half in global memory (absolute column); row ends are relative to
  // the half.
  int csm = 0;
  std::vector<int32_t> csf_a, csf_b, csb_b, csb_a;

  // Triangular-solve streams (entries (x, y), padded to whole chunks):
  // forward over rows 0..n-1, backward over rows n-1..0.
  //   update (y >= 0):              acc -= lu[x] * v[y]
  //   row end (y < 0, y != kNoop):  r = -1 - y; v[r] = v[r] + acc (forward) or
  //                                 (v[r] + acc) * lu[-1-x] (backward, -1-x = diagonal
  //                                 slot holding 1/pivot); acc = 0
  //   no-op (y == kNoop)
  std::vector<int32_t> sf, sb;

  int64_t lu_fma = 0, solve_fma = 0;
  int nnz_l = 0, nnz_u = 0;
};

// Validate a descriptor; returns an empty string when it is consistent.
std::string validate(const fo_mechanism_desc& m);

// Symbolic LU for a given elimination order; returns the multiply-add count
// and fills the row structure when `rows` is non-null.
int64_t symbolic_lu(int n, const std::vector<std::vector<int>>& pattern_rows_perm,
                    std::vector<std::vector<int>>* rows, int* nnz_l, int* nnz_u);

// Build all tables (ordering FO_ORDER_*).
std::string build_tables(const fo_mechanism_desc& m, int ordering, HostTables* t);

}  // namespace fo
