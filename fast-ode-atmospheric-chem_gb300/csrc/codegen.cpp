// Straight-line PTX for one mechanism's factorization and triangular solves.
//
// Why straight-line code. The table-driven kernels (rosenbrock.cuh) spend
// about 40 integer, address and control instructions around every FP64
// multiply-add decoding their streams. Here the pattern is known when the plan
// is made, so every operand is an immediate offset from one base register and
// the instruction stream is the arithmetic itself: one DFMA per update plus
// its share of the operand loads.
//
// The factorization: row blocks of `tile` rows, each cut into column tiles of
// `tile` columns, processed left to right (L tiles, the diagonal tile, U
// tiles). A tile's entries live in registers from assembly to store; every
// pivot k that updates the tile contributes the outer product of its
// multipliers l(i, k) (rows of the tile) and its U row u(k, j) (columns of
// the tile), loaded once per tile: 2t loads for up to t^2 independent FMAs.
// Pivots inside the tile follow in ascending order. Each entry therefore
// receives exactly the updates of the row-by-row elimination, in ascending
// pivot order, with the same operations (fma(-l, u, a); l = a * (1 / pivot);
// 1 / pivot by an IEEE division), so the factors are those of every other
// variant bit for bit. Only structurally nonzero products are emitted: the
// fill pattern's closure (l(i,k) != 0 and u(k,j) != 0 imply (i,j) in the
// pattern) makes each pivot's contribution to a tile a full rectangle.
//
// The solves: blocks of `solve_block` rows; each row sums its terms in
// ascending column order, as the plain variant's loops do, so results match
// that variant bit for bit. In the forward solve a solution value used by
// several rows of a block is loaded once for the block; in the backward
// solve the `solve_keep` values of later blocks used by most rows stay in
// registers for the block and the rest are loaded at each use (holding all of
// them made the register allocator spill about 47 KB per solve to local
// memory, which missed every cache). The transposed solve of the adjoint follows
// the same pattern with rows and columns exchanged.
#include "codegen.h"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "layout.h"

namespace fo {
namespace {

class Ptx {
 public:
  std::string body;
  int next = 1;  // %d0 is alpha

  int reg() { return next++; }

  void line(const char* fmt, ...) __attribute__((format(printf, 2, 3))) {
    char buf[160];
    va_list ap;
    va_start(ap, fmt);
    const int len = vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    body.append("\t");
    body.append(buf, (size_t)std::min<int>(len, (int)sizeof(buf) - 1));
    body.append("\n");
  }
  // value of item `item` of this lane's scratch
  int load(int64_t item) {
    const int r = reg();
    line("ld.global.f64 %%d%d, [%%b+%lld];", r, (long long)(item * 256));
    return r;
  }
  void store(int64_t item, int r) { line("st.global.f64 [%%b+%lld], %%d%d;", (long long)(item * 256), r); }
  int neg(int x) {
    const int r = reg();
    line("neg.f64 %%d%d, %%d%d;", r, x);
    return r;
  }
  int fma(int a, int b, int c) {
    const int r = reg();
    line("fma.rn.f64 %%d%d, %%d%d, %%d%d, %%d%d;", r, a, b, c);
    return r;
  }
  int mul(int a, int b) {
    const int r = reg();
    line("mul.rn.f64 %%d%d, %%d%d, %%d%d;", r, a, b);
    return r;
  }
  int add(int a, int b) {
    const int r = reg();
    line("add.rn.f64 %%d%d, %%d%d, %%d%d;", r, a, b);
    return r;
  }
  int constant(double v) {
    const int r = reg();
    unsigned long long bits;
    static_assert(sizeof(bits) == sizeof(v), "");
    std::memcpy(&bits, &v, sizeof(v));
    line("mov.f64 %%d%d, 0d%016llX;", r, bits);
    return r;
  }
  int recip(int x) {
    const int r = reg();
    line("div.rn.f64 %%d%d, 0d3FF0000000000000, %%d%d;", r, x);
    return r;
  }
};

// Dense map of the LU storage: position of (i, j), or -1.
struct Pattern {
  int n;
  std::vector<int32_t> pos;
  int32_t at(int i, int j) const { return pos[(size_t)i * n + j]; }
};

Pattern pattern_of(const HostTables& t) {
  Pattern P;
  P.n = t.n;
  P.pos.assign((size_t)t.n * t.n, -1);
  for (int i = 0; i < t.n; ++i)
    for (int q = t.lu_row_ptr[i]; q < t.lu_row_ptr[i + 1]; ++q) P.pos[(size_t)i * t.n + t.lu_col[q]] = q;
  return P;
}

// Row blocks [ib_begin, ib_end) of the factorization. A row block reads the
// entries earlier blocks stored and keeps nothing in registers past its end,
// so consecutive ranges can be separate functions called one after another.
void emit_factor(Ptx& x, const HostTables& t, const ScratchLayout& sl, const Pattern& P, int b, int ib_begin,
                 int ib_end, int64_t* nfma) {
  const int n = t.n;
  // Jacobian entry (assembly order) stored at each LU position, or -1
  std::vector<int32_t> jac_at(t.lu_col.size(), -1);
  for (size_t e = 0; e < t.j_lu_pos.size(); ++e) jac_at[t.j_lu_pos[e]] = (int32_t)e;
  const int nb = (n + b - 1) / b;
  std::vector<int> a((size_t)b * b);
  auto A = [&](int i, int j, int i0, int j0) -> int& { return a[(size_t)(i - i0) * b + (j - j0)]; };
  for (int ib = std::max(0, ib_begin); ib < std::min(nb, ib_end); ++ib) {
    const int i0 = ib * b, i1 = std::min(n, i0 + b);
    for (int jb = 0; jb < nb; ++jb) {
      const int j0 = jb * b, j1 = std::min(n, j0 + b);
      bool any = false;
      for (int i = i0; i < i1 && !any; ++i)
        for (int j = j0; j < j1; ++j)
          if (P.at(i, j) >= 0) { any = true; break; }
      if (!any) continue;
      // assembly: -J (or 0 on fill) plus alpha * mass on the diagonal
      for (int i = i0; i < i1; ++i)
        for (int j = j0; j < j1; ++j) {
          const int q = P.at(i, j);
          if (q < 0) continue;
          int v = jac_at[q] >= 0 ? x.load(sl.negj + jac_at[q]) : x.constant(0.0);
          if (i == j) {
            const double m = t.mass[i];
            // alpha * 1 is alpha exactly; any other mass takes the product
            v = x.add(v, m == 1.0 ? 0 : x.mul(0, x.constant(m)));
          }
          A(i, j, i0, j0) = v;
        }
      // pivots left of the tile (and above it): outer products
      const int kmax = std::min(i0, j0);
      std::vector<int> rows, cols, nl(b), u(b);
      for (int k = 0; k < kmax; ++k) {
        rows.clear();
        cols.clear();
        for (int i = i0; i < i1; ++i)
          if (P.at(i, k) >= 0) rows.push_back(i);
        if (rows.empty()) continue;
        for (int j = j0; j < j1; ++j)
          if (P.at(k, j) >= 0) cols.push_back(j);
        if (cols.empty()) continue;
        for (int i : rows) nl[i - i0] = x.neg(x.load(sl.lu + P.at(i, k)));
        for (int j : cols) u[j - j0] = x.load(sl.lu + P.at(k, j));
        for (int i : rows)
          for (int j : cols) {
            if (P.at(i, j) < 0) throw std::logic_error("fill pattern not closed");
            int& r = A(i, j, i0, j0);
            r = x.fma(nl[i - i0], u[j - j0], r);
            ++*nfma;
          }
      }
      if (jb < ib) {
        // an L tile: the multipliers of pivots j0..j1-1, then their updates
        // inside the tile
        for (int k = j0; k < j1; ++k) {
          rows.clear();
          for (int i = i0; i < i1; ++i)
            if (P.at(i, k) >= 0) rows.push_back(i);
          if (rows.empty()) continue;
          const int rk = x.load(sl.lu + P.at(k, k));
          for (int i : rows) {
            int& l = A(i, k, i0, j0);
            l = x.mul(l, rk);
            x.store(sl.lu + P.at(i, k), l);
            nl[i - i0] = x.neg(l);
          }
          for (int j = k + 1; j < j1; ++j) {
            if (P.at(k, j) < 0) continue;
            const int uu = x.load(sl.lu + P.at(k, j));
            for (int i : rows) {
              int& r = A(i, j, i0, j0);
              r = x.fma(nl[i - i0], uu, r);
              ++*nfma;
            }
          }
        }
      } else if (jb == ib) {
        // the diagonal tile: dense elimination inside it
        for (int k = i0; k < i1; ++k) {
          const int rk = x.recip(A(k, k, i0, j0));
          x.store(sl.lu + P.at(k, k), rk);
          for (int j = k + 1; j < i1; ++j)
            if (P.at(k, j) >= 0) x.store(sl.lu + P.at(k, j), A(k, j, i0, j0));
          for (int i = k + 1; i < i1; ++i) {
            if (P.at(i, k) < 0) continue;
            int& l = A(i, k, i0, j0);
            l = x.mul(l, rk);
            x.store(sl.lu + P.at(i, k), l);
            const int nli = x.neg(l);
            for (int j = k + 1; j < i1; ++j) {
              if (P.at(k, j) < 0) continue;
              int& r = A(i, j, i0, j0);
              r = x.fma(nli, A(k, j, i0, j0), r);
              ++*nfma;
            }
          }
        }
      } else {
        // a U tile: rows of the block finish in order and update the rows
        // below them (multipliers from the diagonal tile)
        for (int k = i0; k < i1; ++k) {
          cols.clear();
          for (int j = j0; j < j1; ++j)
            if (P.at(k, j) >= 0) {
              cols.push_back(j);
              x.store(sl.lu + P.at(k, j), A(k, j, i0, j0));
            }
          if (cols.empty()) continue;
          for (int i = k + 1; i < i1; ++i) {
            if (P.at(i, k) < 0) continue;
            const int nli = x.neg(x.load(sl.lu + P.at(i, k)));
            for (int j : cols) {
              int& r = A(i, j, i0, j0);
              r = x.fma(nli, A(k, j, i0, j0), r);
              ++*nfma;
            }
          }
        }
      }
    }
  }
}

void emit_solve(Ptx& x, const HostTables& t, const ScratchLayout& sl, const Pattern& P, int b, int keep) {
  const int n = t.n;
  const int nb = (n + b - 1) / b;
  std::vector<int> xv(n, -1);   // registers of solution values finished in this block
  // forward: x_r -= sum over k < r of L(r, k) x_k, ascending k
  for (int ib = 0; ib < nb; ++ib) {
    const int i0 = ib * b, i1 = std::min(n, i0 + b);
    std::vector<int> acc(b);
    for (int i = i0; i < i1; ++i) acc[i - i0] = x.load(sl.xs + i);
    for (int k = 0; k < i0; ++k) {
      int xk = -1;
      for (int i = i0; i < i1; ++i) {
        const int q = P.at(i, k);
        if (q < 0) continue;
        if (xk < 0) xk = x.load(sl.xs + k);
        acc[i - i0] = x.fma(x.neg(x.load(sl.lu + q)), xk, acc[i - i0]);
      }
    }
    for (int i = i0; i < i1; ++i) {
      for (int k = i0; k < i; ++k) {
        const int q = P.at(i, k);
        if (q >= 0) acc[i - i0] = x.fma(x.neg(x.load(sl.lu + q)), acc[k - i0], acc[i - i0]);
      }
      x.store(sl.xs + i, acc[i - i0]);
    }
  }
  // backward: x_r = (x_r - sum over j > r of U(r, j) x_j) / pivot, ascending j.
  // A row's in-block terms come before its terms in later blocks, so the
  // later blocks' values x_j cannot be summed ahead for the whole block; the
  // `keep` values used by most rows of the block stay in registers from their
  // first load to the end of the block, the others are loaded at each use
  // (keeping every one would hold up to n values live and spill them).
  for (int ib = nb - 1; ib >= 0; --ib) {
    const int i0 = ib * b, i1 = std::min(n, i0 + b);
    std::vector<int> uses(n, 0);
    for (int r = i0; r < i1; ++r)
      for (int q = t.lu_diag[r] + 1; q < t.lu_row_ptr[r + 1]; ++q)
        if (t.lu_col[q] >= i1) ++uses[t.lu_col[q]];
    std::vector<int> order;
    for (int j = i1; j < n; ++j)
      if (uses[j] > 1) order.push_back(j);
    std::stable_sort(order.begin(), order.end(), [&](int u, int v) { return uses[u] > uses[v]; });
    std::vector<char> kept(n, 0);
    for (size_t m = 0; m < order.size() && (int)m < keep; ++m) kept[order[m]] = 1;
    std::vector<int> ext(n, -1);
    for (int r = i1 - 1; r >= i0; --r) {
      int acc = x.load(sl.xs + r);
      for (int q = t.lu_diag[r] + 1; q < t.lu_row_ptr[r + 1]; ++q) {
        const int j = t.lu_col[q];
        int xj;
        if (j < i1) {
          xj = xv[j];
        } else if (kept[j]) {
          if (ext[j] < 0) ext[j] = x.load(sl.xs + j);
          xj = ext[j];
        } else {
          xj = x.load(sl.xs + j);
        }
        acc = x.fma(x.neg(x.load(sl.lu + q)), xj, acc);
      }
      xv[r] = x.mul(acc, x.load(sl.lu + t.lu_diag[r]));
      x.store(sl.xs + r, xv[r]);
    }
  }
}

// The transposed solve A^T x = b in place on the solve vector, the gather
// form of the adjoint's scatter loops (U^T z = b by rows ascending, then
// L^T x = z by rows descending): entry c receives fma(-U(r, c), z_r, .) for
// r ascending, then z_c = . * (1 / pivot_c); later fma(-L(r, c), x_r, .) for r
// descending; the operations of the table-driven kernel in its order.
void emit_solve_t(Ptx& x, const HostTables& t, const ScratchLayout& sl, const Pattern& P, int b) {
  const int n = t.n;
  const int nb = (n + b - 1) / b;
  std::vector<int> xv(n, -1);
  // U^T z = b, columns of U ascending
  for (int ib = 0; ib < nb; ++ib) {
    const int c0 = ib * b, c1 = std::min(n, c0 + b);
    std::vector<int> acc(b);
    for (int c = c0; c < c1; ++c) acc[c - c0] = x.load(sl.xs + c);
    for (int r = 0; r < c0; ++r) {
      int zr = -1;
      for (int c = c0; c < c1; ++c) {
        const int q = P.at(r, c);
        if (q < 0) continue;
        if (zr < 0) zr = x.load(sl.xs + r);
        acc[c - c0] = x.fma(x.neg(x.load(sl.lu + q)), zr, acc[c - c0]);
      }
    }
    for (int c = c0; c < c1; ++c) {
      for (int r = c0; r < c; ++r) {
        const int q = P.at(r, c);
        if (q >= 0) acc[c - c0] = x.fma(x.neg(x.load(sl.lu + q)), xv[r], acc[c - c0]);
      }
      xv[c] = x.mul(acc[c - c0], x.load(sl.lu + P.at(c, c)));
      x.store(sl.xs + c, xv[c]);
    }
  }
  // L^T x = z, columns of L descending
  for (int ib = nb - 1; ib >= 0; --ib) {
    const int c0 = ib * b, c1 = std::min(n, c0 + b);
    std::vector<int> acc(b);
    for (int c = c0; c < c1; ++c) acc[c - c0] = x.load(sl.xs + c);
    for (int r = n - 1; r >= c1; --r) {
      int xr = -1;
      for (int c = c0; c < c1; ++c) {
        const int q = P.at(r, c);
        if (q < 0) continue;
        if (xr < 0) xr = x.load(sl.xs + r);
        acc[c - c0] = x.fma(x.neg(x.load(sl.lu + q)), xr, acc[c - c0]);
      }
    }
    for (int c = c1 - 1; c >= c0; --c) {
      for (int r = c1 - 1; r > c; --r) {
        const int q = P.at(r, c);
        if (q >= 0) acc[c - c0] = x.fma(x.neg(x.load(sl.lu + q)), acc[r - c0], acc[c - c0]);
      }
      x.store(sl.xs + c, acc[c - c0]);
    }
  }
}

// One function whose body dispatches on the mechanism index parameter %m
// to the mechanism's code (`bodies[i]`, all numbered in one register space).
std::string function(const char* name, const char* params, const Ptx& x, const std::vector<std::string>& bodies,
                     const char* prologue) {
  std::string s;
  size_t total = 0;
  for (const auto& b : bodies) total += b.size();
  s.reserve(total + 1024);
  s += ".visible .func ";
  s += name;
  s += "(";
  s += params;
  s += ")\n{\n\t.reg .f64 %d<" + std::to_string(x.next + 1) + ">;\n\t.reg .b64 %p;\n\t.reg .b64 %b;\n"
       "\t.reg .b64 %a;\n\t.reg .b32 %m;\n\t.reg .pred %q;\n";
  s += prologue;
  for (size_t i = 0; i < bodies.size(); ++i) {
    const std::string label = std::string("$") + name + "_m" + std::to_string(i + 1);
    if (i + 1 < bodies.size()) s += "\tsetp.ne.s32 %q, %m, " + std::to_string(i) + ";\n\t@%q bra " + label + ";\n";
    s += bodies[i];
    s += "\tret;\n";
    if (i + 1 < bodies.size()) s += label + ":\n";
  }
  s += "}\n";
  return s;
}

// The factorization: every piece of every mechanism as its own function
// (fo_gen_factor_m<m>_p<k>: base, alpha), then fo_gen_factor(base, alpha,
// mech), which calls mechanism mech's pieces in order. Separate functions
// keep each compilation unit of the register allocator and scheduler small.
std::string factor_functions(const std::vector<std::vector<Ptx>>& pieces) {
  std::string out;
  for (size_t m = 0; m < pieces.size(); ++m)
    for (size_t k = 0; k < pieces[m].size(); ++k) {
      const Ptx& x = pieces[m][k];
      const std::string name = "fo_gen_factor_m" + std::to_string(m) + "_p" + std::to_string(k);
      out.reserve(out.size() + x.body.size() + 512);
      out += ".func " + name + "(.param .b64 " + name + "_base, .param .b64 " + name + "_alpha)\n{\n";
      out += "\t.reg .f64 %d<" + std::to_string(x.next + 1) + ">;\n\t.reg .b64 %p;\n\t.reg .b64 %b;\n"
             "\t.reg .b64 %a;\n";
      out += "\tld.param.b64 %p, [" + name + "_base];\n\tld.param.b64 %a, [" + name + "_alpha];\n"
             "\tmov.b64 %d0, %a;\n\tcvta.to.global.u64 %b, %p;\n";
      out += x.body;
      out += "\tret;\n}\n\n";
    }
  out += ".visible .func fo_gen_factor(.param .b64 fo_gen_factor_base, .param .b64 fo_gen_factor_alpha, "
         ".param .b32 fo_gen_factor_mech)\n{\n\t.reg .b64 %p;\n\t.reg .b64 %a;\n\t.reg .b32 %m;\n"
         "\t.reg .pred %q;\n\tld.param.b64 %p, [fo_gen_factor_base];\n\tld.param.b64 %a, [fo_gen_factor_alpha];\n"
         "\tld.param.b32 %m, [fo_gen_factor_mech];\n";
  for (size_t m = 0; m < pieces.size(); ++m) {
    const std::string label = "$fo_gen_factor_m" + std::to_string(m + 1);
    if (m + 1 < pieces.size()) out += "\tsetp.ne.s32 %q, %m, " + std::to_string(m) + ";\n\t@%q bra " + label + ";\n";
    for (size_t k = 0; k < pieces[m].size(); ++k)
      out += "\t{\n\t.param .b64 fo_arg_base;\n\t.param .b64 fo_arg_alpha;\n\tst.param.b64 [fo_arg_base], %p;\n"
             "\tst.param.b64 [fo_arg_alpha], %a;\n\tcall.uni fo_gen_factor_m" + std::to_string(m) + "_p" +
             std::to_string(k) + ", (fo_arg_base, fo_arg_alpha);\n\t}\n";
    out += "\tret;\n";
    if (m + 1 < pieces.size()) out += label + ":\n";
  }
  out += "}\n";
  return out;
}

}  // namespace

std::string generate_ptx(const std::vector<const HostTables*>& ts, const std::vector<GenOptions>& os,
                         int64_t* fma_count) {
  if (ts.empty() || os.size() != ts.size()) throw std::invalid_argument("one set of options per mechanism");
  for (const GenOptions& o : os)
    if (o.tile < 1 || o.tile > 16 || o.solve_block < 1 || o.solve_block > 64 || o.solve_keep < 0 ||
        o.piece_lines < 1)
      throw std::invalid_argument("generation options out of range");
  Ptx s, st;
  std::vector<std::string> sb, tb;
  // the factorization of mechanism m: pieces[m][k] = the k-th function
  std::vector<std::vector<Ptx>> pieces(ts.size());
  int64_t total = 0;
  for (size_t m = 0; m < ts.size(); ++m) {
    const HostTables* t = ts[m];
    const GenOptions& o = os[m];
    const ScratchLayout sl = layout_of(*t);
    const Pattern P = pattern_of(*t);
    // consecutive row blocks up to about o.piece_lines instructions each
    const int nb = (t->n + o.tile - 1) / o.tile;
    std::vector<size_t> lines(nb);
    for (int ib = 0; ib < nb; ++ib) {
      Ptx probe;
      int64_t ignored = 0;
      emit_factor(probe, *t, sl, P, o.tile, ib, ib + 1, &ignored);
      lines[ib] = (size_t)std::count(probe.body.begin(), probe.body.end(), '\n');
    }
    int64_t nfma = 0;
    for (int ib = 0; ib < nb;) {
      int end = ib + 1;
      size_t sum = lines[ib];
      while (end < nb && sum + lines[end] <= (size_t)o.piece_lines) sum += lines[end++];
      pieces[m].emplace_back();
      emit_factor(pieces[m].back(), *t, sl, P, o.tile, ib, end, &nfma);
      ib = end;
    }
    if (nfma != t->lu_fma) throw std::logic_error("generated factorization does not match the symbolic count");
    total += nfma;
    emit_solve(s, *t, sl, P, o.solve_block, o.solve_keep);
    sb.push_back(std::move(s.body));
    s.body.clear();
    emit_solve_t(st, *t, sl, P, o.solve_block);
    tb.push_back(std::move(st.body));
    st.body.clear();
  }
  if (fma_count) *fma_count = total;
  std::string out = ".version 9.0\n.target sm_103a\n.address_size 64\n\n";
  out += factor_functions(pieces);
  out += "\n";
  out += function("fo_gen_solve", ".param .b64 fo_gen_solve_base, .param .b32 fo_gen_solve_mech", s, sb,
                  "\tld.param.b64 %p, [fo_gen_solve_base];\n\tld.param.b32 %m, [fo_gen_solve_mech];\n"
                  "\tcvta.to.global.u64 %b, %p;\n");
  out += "\n";
  out += function("fo_gen_solve_t", ".param .b64 fo_gen_solve_t_base, .param .b32 fo_gen_solve_t_mech", st, tb,
                  "\tld.param.b64 %p, [fo_gen_solve_t_base];\n\tld.param.b32 %m, [fo_gen_solve_t_mech];\n"
                  "\tcvta.to.global.u64 %b, %p;\n");
  return out;
}

std::string generate_ptx(const HostTables& t, const GenOptions& o, int64_t* fma_count) {
  return generate_ptx(std::vector<const HostTables*>{&t}, std::vector<GenOptions>{o}, fma_count);
}

}  // namespace fo
