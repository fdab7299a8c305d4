// Symbolic analysis for the pivot-free batched sparse LU.
//
// The reference factors alpha*M - J of a whole group with SuperLU and the
// MMD_AT_PLUS_A column ordering, from scratch on every attempt
// (fastode/linalg.py:70-78), with partial pivoting. Here the ordering and the
// fill pattern are computed once per mechanism: the same pattern serves every
// cell and every attempt, so the device runs a fixed, branch-free elimination.
// Pivoting is dropped, as MICM's LuDecompositionMozartInPlace (the reference's
// validated baseline, validation/micm_scenario.cpp:46-51) drops it; the stage
// matrix of a stiff chemistry system is dominated by its diagonal.
#include "symbolic.h"

#include <algorithm>
#include <climits>
#include <cstring>
#include <numeric>
#include <queue>
#include <set>

namespace fo {

std::string validate(const fo_mechanism_desc& m) {
  if (m.n <= 0) return "n must be positive";
  if (m.R < 0) return "R must be non-negative";
  if (m.P <= 0) return "P must be positive";
  if (m.nnz < m.n) return "the Jacobian pattern must hold the diagonal";
  if (!m.pat_rows || !m.pat_cols) return "missing Jacobian pattern";
  if (m.R > 0 && (!m.react || !m.s_indptr || !m.j_indptr)) return "missing reaction tables";
  if (!m.s_indptr) return "missing stoichiometry";
  for (int64_t q = 0; q < (int64_t)m.R * m.P; ++q)
    if (m.react[q] < 0 || m.react[q] > m.n) return "reactant index out of range";
  if (m.s_indptr[0] != 0) return "stoichiometry indptr must start at 0";
  for (int i = 0; i < m.n; ++i)
    if (m.s_indptr[i + 1] < m.s_indptr[i]) return "stoichiometry indptr must be non-decreasing";
  for (int q = 0; q < m.s_indptr[m.n]; ++q)
    if (m.s_idx[q] < 0 || m.s_idx[q] >= m.R) return "stoichiometry reaction index out of range";
  std::vector<char> diag(m.n, 0);
  for (int e = 0; e < m.nnz; ++e) {
    if (m.pat_rows[e] < 0 || m.pat_rows[e] >= m.n || m.pat_cols[e] < 0 || m.pat_cols[e] >= m.n)
      return "pattern index out of range";
    if (m.pat_rows[e] == m.pat_cols[e]) diag[m.pat_rows[e]] = 1;
  }
  for (int i = 0; i < m.n; ++i)
    if (!diag[i]) return "the Jacobian pattern must hold every diagonal entry";
  if (m.j_indptr) {
    if (m.j_indptr[0] != 0) return "Jacobian map indptr must start at 0";
    for (int e = 0; e < m.nnz; ++e)
      if (m.j_indptr[e + 1] < m.j_indptr[e]) return "Jacobian map indptr must be non-decreasing";
    for (int q = 0; q < m.j_indptr[m.nnz]; ++q)
      if (m.j_idx[q] < 0 || m.j_idx[q] >= m.R * m.P) return "Jacobian map column out of range";
  }
  return "";
}

int64_t symbolic_lu(int n, const std::vector<std::vector<int>>& pat, std::vector<std::vector<int>>* rows,
                    int* nnz_l, int* nnz_u) {
  // Row-by-row (up-looking) symbolic elimination: row i's final pattern is its
  // own pattern united with U(k) for every k < i that ends up in L(i).
  std::vector<std::vector<int>> U(n);
  std::vector<int> mark(n, -1);
  int64_t fma = 0;
  int nl = 0, nu = 0;
  if (rows) rows->assign(n, {});
  for (int i = 0; i < n; ++i) {
    std::vector<int> members;
    std::priority_queue<int, std::vector<int>, std::greater<int>> lower;
    auto add = [&](int c) {
      if (mark[c] == i) return;
      mark[c] = i;
      members.push_back(c);
      if (c < i) lower.push(c);
    };
    add(i);
    for (int c : pat[i]) add(c);
    while (!lower.empty()) {
      int k = lower.top();
      lower.pop();
      fma += (int64_t)U[k].size();
      for (int j : U[k]) add(j);
    }
    std::sort(members.begin(), members.end());
    for (int c : members) {
      if (c < i) ++nl;
      if (c > i) {
        ++nu;
        U[i].push_back(c);
      }
    }
    if (rows) (*rows)[i] = members;
  }
  if (nnz_l) *nnz_l = nl;
  if (nnz_u) *nnz_u = nu;
  return fma;
}

namespace {

struct Bitset {
  int words = 0;
  std::vector<uint64_t> bits;
  void init(int n, int count) {
    words = (n + 63) / 64;
    bits.assign((size_t)words * count, 0);
  }
  uint64_t* row(int i) { return bits.data() + (size_t)i * words; }
};

int popcnt(uint64_t x) { return __builtin_popcountll(x); }

// Greedy elimination on the symmetric graph of A + A^T. mode 0: minimum
// degree; mode 1: minimum fill among the `window` lowest-degree vertices.
// Ties go to the lowest degree, then the lowest index.
std::vector<int> greedy_order(int n, const std::vector<std::vector<int>>& adj_in, int mode, int window) {
  Bitset g;
  g.init(n, n);
  for (int i = 0; i < n; ++i)
    for (int j : adj_in[i])
      if (i != j) {
        g.row(i)[j / 64] |= 1ull << (j % 64);
        g.row(j)[i / 64] |= 1ull << (i % 64);
      }
  std::vector<char> alive(n, 1);
  std::vector<int> degree(n, 0), order;
  order.reserve(n);
  auto deg = [&](int v) {
    int d = 0;
    uint64_t* r = g.row(v);
    for (int w = 0; w < g.words; ++w) d += popcnt(r[w]);
    return d;
  };
  for (int v = 0; v < n; ++v) degree[v] = deg(v);
  std::vector<int> nb;
  for (int step = 0; step < n; ++step) {
    int best = -1;
    if (mode == 0) {
      for (int v = 0; v < n; ++v)
        if (alive[v] && (best < 0 || degree[v] < degree[best])) best = v;
    } else {
      std::vector<int> cand;
      for (int v = 0; v < n; ++v)
        if (alive[v]) cand.push_back(v);
      std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) { return degree[a] < degree[b]; });
      if ((int)cand.size() > window) cand.resize(window);
      int64_t best_fill = -1;
      for (int v : cand) {
        uint64_t* rv = g.row(v);
        int64_t fill = 0;
        for (int w = 0; w < g.words; ++w) {
          uint64_t x = rv[w];
          while (x) {
            int a = w * 64 + __builtin_ctzll(x);
            x &= x - 1;
            uint64_t* ra = g.row(a);
            for (int u = 0; u < g.words; ++u) fill += popcnt(rv[u] & ~ra[u]);
            fill -= 1;  // a itself
          }
        }
        if (best < 0 || fill < best_fill || (fill == best_fill && degree[v] < degree[best])) {
          best = v;
          best_fill = fill;
        }
      }
    }
    order.push_back(best);
    alive[best] = 0;
    nb.clear();
    uint64_t* rb = g.row(best);
    for (int w = 0; w < g.words; ++w) {
      uint64_t x = rb[w];
      while (x) {
        nb.push_back(w * 64 + __builtin_ctzll(x));
        x &= x - 1;
      }
    }
    for (int a : nb) {
      uint64_t* ra = g.row(a);
      for (int w = 0; w < g.words; ++w) ra[w] |= rb[w];
      ra[a / 64] &= ~(1ull << (a % 64));
      ra[best / 64] &= ~(1ull << (best % 64));
    }
    std::fill(rb, rb + g.words, 0ull);
    for (int a : nb) degree[a] = deg(a);
  }
  return order;
}

std::vector<std::vector<int>> permuted_pattern(const fo_mechanism_desc& m, const std::vector<int>& iperm) {
  std::vector<std::vector<int>> pat(m.n);
  for (int e = 0; e < m.nnz; ++e) pat[iperm[m.pat_rows[e]]].push_back(iperm[m.pat_cols[e]]);
  return pat;
}

int64_t cost_of(const fo_mechanism_desc& m, const std::vector<int>& order) {
  std::vector<int> iperm(m.n);
  for (int p = 0; p < m.n; ++p) iperm[order[p]] = p;
  return symbolic_lu(m.n, permuted_pattern(m, iperm), nullptr, nullptr, nullptr);
}

// The cost of an elimination order for the local search below: the
// elimination's FMAs plus kEntryWeight per LU entry, since every attempt also
// runs three stage solves that touch each entry once. With weight 4 the search
// on the 210-species mechanism keeps its FMA count and finds orders with
// about 9% fewer entries; larger weights trade FMAs for entries.
// Counted by bitset symbolic elimination: row i's pattern is its own united
// with U(k) for each k < i in it, taken in increasing k (merging U(k) only
// adds columns above k, so one ascending scan finds them all).
constexpr int64_t kEntryWeight = 4;

class FmaCounter {
 public:
  explicit FmaCounter(const fo_mechanism_desc& m) : n_(m.n), words_((m.n + 63) / 64), nnz_(m.nnz), pat_(m.n) {
    for (int e = 0; e < m.nnz; ++e) pat_[m.pat_rows[e]].push_back((int)m.pat_cols[e]);
    for (int i = 0; i < n_; ++i) pat_[i].push_back(i);
    rows_.assign((size_t)n_ * words_, 0);
    upper_.assign((size_t)n_ * words_, 0);
    ucount_.assign(n_, 0);
    pos_.assign(n_, 0);
  }
  // Stops early, returning a count >= limit, once the count reaches limit.
  int64_t count(const std::vector<int>& order, int64_t limit) {
    const int W = words_;
    for (int p = 0; p < n_; ++p) pos_[order[p]] = p;
    std::fill(rows_.begin(), rows_.end(), 0ull);
    for (int v = 0; v < n_; ++v) {
      uint64_t* r = &rows_[(size_t)pos_[v] * W];
      for (int c : pat_[v]) r[pos_[c] >> 6] |= 1ull << (pos_[c] & 63);
    }
    int64_t fma = 0;
    for (int i = 0; i < n_; ++i) {
      uint64_t* row = &rows_[(size_t)i * W];
      const int iw = i >> 6, ib = i & 63;
      for (int w = 0; w <= iw; ++w) {
        const uint64_t below_i = w < iw ? ~0ull : ((1ull << ib) - 1);
        uint64_t unseen = ~0ull;
        for (;;) {
          const uint64_t x = row[w] & below_i & unseen;
          if (!x) break;
          const int b = __builtin_ctzll(x);
          const int k = w * 64 + b;
          unseen = b == 63 ? 0ull : ~((2ull << b) - 1);
          fma += ucount_[k];
          const uint64_t* uk = &upper_[(size_t)k * W];
          for (int u = w; u < W; ++u) row[u] |= uk[u];
        }
      }
      uint64_t* ui = &upper_[(size_t)i * W];
      int c = 0;
      for (int u = 0; u < W; ++u) {
        const uint64_t x = u < iw ? 0ull : u > iw ? row[u] : (ib == 63 ? 0ull : row[u] & ~((2ull << ib) - 1));
        ui[u] = x;
        c += popcnt(x);
      }
      ucount_[i] = c;
      int entries = 0;
      for (int u = 0; u < W; ++u) entries += popcnt(row[u]);
      fma += kEntryWeight * entries;
      if (fma >= limit) return fma;
    }
    return fma;
  }
  // Word operations of one evaluation, for sizing the search.
  int64_t work(const std::vector<int>& order) {
    count(order, INT64_MAX);
    int64_t l = 0;
    for (int i = 0; i < n_; ++i) l += ucount_[i];
    return (int64_t)n_ * words_ + nnz_ + l * words_;
  }

 private:
  int n_, words_;
  int64_t nnz_;
  std::vector<std::vector<int>> pat_;
  std::vector<uint64_t> rows_, upper_;
  std::vector<int> ucount_, pos_;
};

// splitmix64: a fixed, portable pseudo-random stream.
struct SplitMix {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  int below(int n) { return (int)(next() % (uint64_t)n); }
};

// Local search on the elimination order by threshold accepting: move one
// species to another position and keep the move while the cost above stays
// below the current cost plus a threshold that falls linearly from 0.3% of
// the starting cost to zero. The greedy orders above minimise fill one
// elimination at a time; on the random-graph patterns of large mechanisms
// this finds orders with about half their FMAs. Integer arithmetic and a
// fixed seed make the order the same on every host. The number of moves is
// capped by an operation budget (about a second for 210 species). Returns
// the best order found; *improved tells whether it is cheaper than start.
std::vector<int> refine_order(const fo_mechanism_desc& m, const std::vector<int>& start, bool* improved) {
  const int n = m.n;
  *improved = false;
  if (n < 3) return start;
  FmaCounter counter(m);
  const int64_t kWorkBudget = 600000000;
  // the operation budget bounds the host time for large mechanisms; below a
  // few hundred moves the search would not get anywhere, so it is skipped
  const int64_t moves = std::min<int64_t>(20000, kWorkBudget / std::max<int64_t>(1, counter.work(start)));
  if (moves < 200) return start;
  std::vector<int> order = start, best = start, trial(n);
  int64_t cur = counter.count(start, INT64_MAX), best_cost = cur;
  const int64_t start_cost = cur;
  const int64_t t0 = cur * 3 / 1000;
  SplitMix rng{0x5eedf00dull};
  for (int64_t e = 0; e < moves; ++e) {
    const int64_t threshold = t0 - t0 * e / moves;
    const int i = rng.below(n), j = rng.below(n);
    if (i == j) continue;
    trial = order;
    const int v = trial[i];
    if (i < j)
      for (int q = i; q < j; ++q) trial[q] = trial[q + 1];
    else
      for (int q = i; q > j; --q) trial[q] = trial[q - 1];
    trial[j] = v;
    const int64_t c = counter.count(trial, cur + threshold);
    if (c < cur + threshold) {
      order.swap(trial);
      cur = c;
      if (cur < best_cost) {
        best_cost = cur;
        best = order;
      }
    }
  }
  *improved = best_cost < start_cost;
  return best;
}

}  // namespace

// The compact variant's tables (see HostTables), built from the LU structure
// and the Jacobian's positions in it.
void build_compact(HostTables* t) {
  const int n = t->n;
  t->cs_split.assign(n, 0);
  t->cs_jsplit.assign(n, 0);
  t->ce_ptr.assign(1, 0);
  t->cep.clear();
  t->cmax_half = 0;
  if ((int64_t)t->lu_col.size() > 65536 || t->max_row_len >= 0x7ffe) {
    t->ce_ptr.clear();
    return;
  }
  std::vector<int> slot_of(n, -1);
  std::vector<int64_t> touched(n, -1);
  auto entries = [&]() { return (int64_t)t->cep.size(); };
  auto pad = [&]() {
    while (entries() % kStreamChunk != 0) t->cep.push_back(0x7fffu);
  };
  auto pad_chunk = [&]() {
    t->cep.push_back(0x7fffu);
    pad();
  };
  // an entry that touches `slot` (relative to the pass) may not share a chunk
  // with an earlier update of it
  auto place = [&](int slot) {
    while (touched[slot] >= entries() / kStreamChunk) pad_chunk();
  };
  // A multiplier's updates, in any order (each touches its own slot, and a
  // slot still receives its updates in multiplier order, so the factors do not
  // change): each next entry is the first pending update whose slot the
  // current chunk has not touched; the chunk is padded only when none is left.
  std::vector<std::pair<int, int>> group;  // (slot relative to the pass, LU position of the U entry)
  auto emit_group = [&]() {
    size_t done = 0;
    while (done < group.size()) {
      const int64_t chunk = entries() / kStreamChunk;
      size_t pick = group.size();
      for (size_t i = done; i < group.size(); ++i)
        if (touched[group[i].first] < chunk) {
          pick = i;
          break;
        }
      if (pick == group.size()) {
        pad_chunk();
        continue;
      }
      std::swap(group[done], group[pick]);
      const int y = group[done].first, u = group[done].second;
      touched[y] = chunk;
      t->cep.push_back(((uint32_t)u << 16) | (uint32_t)y);
      ++done;
    }
    group.clear();
  };
  for (int r = 0; r < n; ++r) {
    const int q0 = t->lu_row_ptr[r], len = t->lu_row_ptr[r + 1] - q0, dg = t->lu_diag[r];
    const int split = (len + 1) / 2;
    t->cs_split[r] = split;
    t->cmax_half = std::max(t->cmax_half, std::max(split, len - split));
    for (int q = q0; q < q0 + len; ++q) slot_of[t->lu_col[q]] = q - q0;
    for (int pass = 0; pass < 2; ++pass) {
      const int base = pass ? split : 0, cnt = pass ? len - split : split;
      for (int s = 0; s < cnt; ++s) touched[s] = -2;
      for (int q = q0; q < dg; ++q) {
        const int k = t->lu_col[q], ks = q - q0;
        const bool in_a = ks < split;
        if (pass == 0 && !in_a) break;                       // pass A: the leading multipliers only
        bool opened = false;
        if (pass == 0 || !in_a) {                            // the pass that makes l_rk
          place(ks - base);
          t->cep.push_back(((uint32_t)t->lu_diag[k] << 16) | 0x8000u | (uint32_t)(ks - base));
          opened = true;
        }
        for (int u = t->lu_diag[k] + 1; u < t->lu_row_ptr[k + 1]; ++u) {
          const int y = slot_of[t->lu_col[u]];
          if ((y >= split) != (pass == 1)) continue;         // the other pass's column
          if (!opened) {                                     // pass B reloads a multiplier of pass A
            t->cep.push_back(((uint32_t)q << 16) | kReloadSlot);
            opened = true;
          }
          group.push_back({y - base, u});
        }
        emit_group();
      }
      pad();
      t->ce_ptr.push_back((int32_t)t->cep.size());
    }
    int e = t->j_row_ptr[r];
    while (e < t->j_row_ptr[r + 1] && t->j_lu_pos[e] - q0 < split) ++e;
    t->cs_jsplit[r] = e;
  }
  // the split solves
  const int m = (n + 1) / 2;
  t->csm = m;
  auto finish = [](std::vector<int32_t>* st) {
    while ((st->size() / 2) % kStreamChunk != 0) {
      st->push_back(-1);
      st->push_back(kNoop);
    }
  };
  auto operand = [&](int col, int half_base, int half_end) {
    return (col >= half_base && col < half_end) ? col - half_base : (col | kGlobalOperand);
  };
  for (std::vector<int32_t>* st : {&t->csf_a, &t->csf_b, &t->csb_b, &t->csb_a}) st->clear();
  for (int r = 0; r < n; ++r) {                            // forward: L y = b
    std::vector<int32_t>* st = r < m ? &t->csf_a : &t->csf_b;
    const int hb = r < m ? 0 : m, he = r < m ? m : n;
    for (int q = t->lu_row_ptr[r]; q < t->lu_diag[r]; ++q) {
      st->push_back(q);
      st->push_back(operand(t->lu_col[q], hb, he));
    }
    st->push_back(-1);
    st->push_back(-1 - (r - hb));
  }
  for (int r = n - 1; r >= 0; --r) {                       // backward: U x = y
    std::vector<int32_t>* st = r >= m ? &t->csb_b : &t->csb_a;
    const int hb = r < m ? 0 : m, he = r < m ? m : n;
    for (int q = t->lu_diag[r] + 1; q < t->lu_row_ptr[r + 1]; ++q) {
      st->push_back(q);
      st->push_back(operand(t->lu_col[q], hb, he));
    }
    st->push_back(-1 - t->lu_diag[r]);
    st->push_back(-1 - (r - hb));
  }
  for (std::vector<int32_t>* st : {&t->csf_a, &t->csf_b, &t->csb_b, &t->csb_a}) finish(st);
}

std::string build_tables(const fo_mechanism_desc& m, int ordering, HostTables* t) {
  std::string err = validate(m);
  if (!err.empty()) return err;
  const int n = m.n, R = m.R, P = m.P;
  t->n = n;
  t->R = R;
  t->P = P;
  t->nnz = m.nnz;

  // symmetric structure for the orderings
  std::vector<std::vector<int>> adj(n);
  for (int e = 0; e < m.nnz; ++e) adj[m.pat_rows[e]].push_back((int)m.pat_cols[e]);

  std::vector<int> natural(n);
  std::iota(natural.begin(), natural.end(), 0);
  std::vector<std::pair<int, std::vector<int>>> cands;
  const bool every = ordering == FO_ORDER_AUTO || ordering == FO_ORDER_REFINED;
  if (ordering == FO_ORDER_NATURAL || every) cands.push_back({FO_ORDER_NATURAL, natural});
  if (ordering == FO_ORDER_MIN_DEGREE || every) cands.push_back({FO_ORDER_MIN_DEGREE, greedy_order(n, adj, 0, 0)});
  if (ordering == FO_ORDER_MIN_FILL || every) {
    cands.push_back({FO_ORDER_MIN_FILL, greedy_order(n, adj, 1, n <= 400 ? n : 32)});
    if (every && n > 8) cands.push_back({FO_ORDER_MIN_FILL, greedy_order(n, adj, 1, 8)});
  }
  if (cands.empty()) return "unknown ordering";
  int best = 0;
  int64_t best_cost = -1;
  for (size_t c = 0; c < cands.size(); ++c) {
    int64_t cost = cost_of(m, cands[c].second);
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      best = (int)c;
    }
  }
  t->ordering = cands[best].first;
  std::vector<int> chosen = cands[best].second;
  if (every) {
    bool improved = false;
    std::vector<int> refined = refine_order(m, chosen, &improved);
    if (improved || ordering == FO_ORDER_REFINED) {
      chosen = refined;
      t->ordering = FO_ORDER_REFINED;
    }
  }
  t->perm.assign(chosen.begin(), chosen.end());
  t->iperm.assign(n, 0);
  for (int p = 0; p < n; ++p) t->iperm[t->perm[p]] = p;

  t->mass.assign(n, 1.0);
  if (m.mass)
    for (int p = 0; p < n; ++p) t->mass[p] = m.mass[t->perm[p]];

  // rates
  t->react.assign((size_t)R * P, n);
  for (int j = 0; j < R; ++j)
    for (int p = 0; p < P; ++p) {
      int64_t s = m.react[(size_t)j * P + p];
      t->react[(size_t)j * P + p] = s == n ? n : t->iperm[s];
    }
  // stoichiometry rows in permuted order
  t->s_ptr.assign(1, 0);
  t->s_rxn.clear();
  t->s_val.clear();
  for (int p = 0; p < n; ++p) {
    int i = t->perm[p];
    for (int q = m.s_indptr[i]; q < m.s_indptr[i + 1]; ++q) {
      t->s_rxn.push_back(m.s_idx[q]);
      t->s_val.push_back(m.s_val[q]);
    }
    t->s_ptr.push_back((int32_t)t->s_rxn.size());
  }

  // S by reactions (for the adjoint's S^T v)
  {
    std::vector<std::vector<std::pair<int, double>>> cols(R);
    for (int p = 0; p < n; ++p)
      for (int q = t->s_ptr[p]; q < t->s_ptr[p + 1]; ++q) cols[t->s_rxn[q]].push_back({p, t->s_val[q]});
    t->st_ptr.assign(1, 0);
    t->st_sp.clear();
    t->st_val.clear();
    for (int j = 0; j < R; ++j) {
      for (auto& e : cols[j]) {
        t->st_sp.push_back(e.first);
        t->st_val.push_back(e.second);
      }
      t->st_ptr.push_back((int32_t)t->st_sp.size());
    }
  }

  // LU structure
  std::vector<std::vector<int>> pat = permuted_pattern(m, t->iperm);
  std::vector<std::vector<int>> rows;
  t->lu_fma = symbolic_lu(n, pat, &rows, &t->nnz_l, &t->nnz_u);
  t->solve_fma = (int64_t)t->nnz_l + t->nnz_u;
  t->lu_row_ptr.assign(1, 0);
  t->lu_diag.assign(n, 0);
  t->lu_col.clear();
  for (int r = 0; r < n; ++r) {
    for (int c : rows[r]) {
      if (c == r) t->lu_diag[r] = (int32_t)t->lu_col.size();
      t->lu_col.push_back(c);
    }
    t->lu_row_ptr.push_back((int32_t)t->lu_col.size());
  }

  // elimination stream, row by row, each row padded to whole chunks; the
  // targets are slots of the row's own pattern (its position minus the row
  // start), so the work row needs max_row_len entries, not n
  t->el_ptr.assign(1, 0);
  t->el.clear();
  t->max_row_len = 0;
  // Every chunk is hazard-free over a window of kHazardWindow chunks: no slot
  // is updated twice in a chunk, and no entry (update or multiplier) touches a
  // slot that an earlier entry of the same chunk (or, with a window of two, of
  // the previous chunk) updated. The device then reads a chunk's work-row
  // values at once, runs its updates as independent FMAs (only the multipliers
  // chain them) and writes them back: FP64 latency overlaps instead of
  // serializing every read-modify-write.
  std::vector<int> slot_of(n, -1);
  std::vector<int64_t> touched(n, -1);  // absolute chunk that last updated a slot
  auto entries = [&]() { return (int64_t)(t->el.size() / 2); };
  auto pad = [&]() {
    while (entries() % kStreamChunk != 0) {
      t->el.push_back(-1);
      t->el.push_back(-1);
    }
  };
  // close the current chunk (a whole no-op chunk when it is empty)
  auto pad_chunk = [&]() {
    t->el.push_back(-1);
    t->el.push_back(-1);
    pad();
  };
  for (int r = 0; r < n; ++r) {
    const int q0 = t->lu_row_ptr[r];
    t->max_row_len = std::max(t->max_row_len, t->lu_row_ptr[r + 1] - q0);
    for (int q = q0; q < t->lu_row_ptr[r + 1]; ++q) {
      slot_of[t->lu_col[q]] = q - q0;
      touched[q - q0] = -2;                         // the row's slots start unwritten
    }
    for (int q = q0; q < t->lu_diag[r]; ++q) {
      const int k = t->lu_col[q];
      const int ym = q - q0;                        // the multiplier reads slot ym
      while (touched[ym] >= entries() / kStreamChunk - (kHazardWindow - 1)) pad_chunk();
      t->el.push_back(-1 - t->lu_diag[k]);
      t->el.push_back(ym);
      for (int u = t->lu_diag[k] + 1; u < t->lu_row_ptr[k + 1]; ++u) {
        const int y = slot_of[t->lu_col[u]];
        while (touched[y] >= entries() / kStreamChunk - (kHazardWindow - 1)) pad_chunk();
        touched[y] = entries() / kStreamChunk;
        t->el.push_back(u);
        t->el.push_back(y);
      }
    }
    pad();
    t->el_ptr.push_back((int32_t)(t->el.size() / 2));
  }

  // packed copy of the elimination stream
  t->elp.clear();
  if ((int64_t)t->lu_col.size() <= 65536 && t->max_row_len < 0x7fff) {
    t->elp.reserve(t->el.size() / 2);
    for (size_t e = 0; e < t->el.size(); e += 2) {
      const int32_t x = t->el[e], y = t->el[e + 1];
      uint32_t word;
      if (x >= 0) word = ((uint32_t)x << 16) | (uint32_t)y;                       // update
      else if (y >= 0) word = ((uint32_t)(-1 - x) << 16) | 0x8000u | (uint32_t)y;  // multiplier
      else word = 0x7fffu;                                                        // padding
      t->elp.push_back(word);
    }
  }

  // triangular-solve streams (one flat sequence each, padded at the end)
  t->sf.clear();
  t->sb.clear();
  for (int r = 0; r < n; ++r) {
    for (int q = t->lu_row_ptr[r]; q < t->lu_diag[r]; ++q) {
      t->sf.push_back(q);
      t->sf.push_back(t->lu_col[q]);
    }
    t->sf.push_back(-1);
    t->sf.push_back(-1 - r);
  }
  for (int r = n - 1; r >= 0; --r) {
    for (int q = t->lu_diag[r] + 1; q < t->lu_row_ptr[r + 1]; ++q) {
      t->sb.push_back(q);
      t->sb.push_back(t->lu_col[q]);
    }
    t->sb.push_back(-1 - t->lu_diag[r]);
    t->sb.push_back(-1 - r);
  }
  for (std::vector<int32_t>* s : {&t->sf, &t->sb})
    while ((s->size() / 2) % kStreamChunk != 0) {
      s->push_back(-1);
      s->push_back(kNoop);
    }

  // Jacobian entries in assembly order
  std::vector<std::vector<std::pair<int, int>>> by_row(n);  // (perm col, original entry)
  for (int e = 0; e < m.nnz; ++e)
    by_row[t->iperm[m.pat_rows[e]]].push_back({t->iperm[m.pat_cols[e]], e});
  t->j_row_ptr.assign(1, 0);
  t->j_col.clear();
  t->j_src.clear();
  t->j_lu_pos.clear();
  t->jt_ptr.assign(1, 0);
  t->jt_idx.clear();
  t->jt_val.clear();
  for (int r = 0; r < n; ++r) {
    std::sort(by_row[r].begin(), by_row[r].end());
    for (auto& ce : by_row[r]) {
      int c = ce.first, e = ce.second;
      t->j_col.push_back(c);
      t->j_src.push_back(e);
      auto b = t->lu_col.begin() + t->lu_row_ptr[r], en = t->lu_col.begin() + t->lu_row_ptr[r + 1];
      auto it = std::lower_bound(b, en, c);
      t->j_lu_pos.push_back((int32_t)(it - t->lu_col.begin()));
      if (m.j_indptr)
        for (int q = m.j_indptr[e]; q < m.j_indptr[e + 1]; ++q) {
          t->jt_idx.push_back(m.j_idx[q]);
          t->jt_val.push_back(-m.j_val[q]);
        }
      t->jt_ptr.push_back((int32_t)t->jt_idx.size());
    }
    t->j_row_ptr.push_back((int32_t)t->j_col.size());
  }
  build_compact(t);
  return "";
}

}  // namespace fo
