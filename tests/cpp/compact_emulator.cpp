// Host emulation of the compact factorization and split solves over the
// tables symbolic.cpp builds, for one cell: checks every table against the
// plain row-by-row LU (bit for bit) and triangular solves (to roundoff)
// before any of it runs on a GPU. Reads the mechanism descriptor from a
// binary file written by the test (arrays as int64 count + raw data).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "symbolic.h"

template <typename T>
std::vector<T> read_array(FILE* f) {
  int64_t n = 0;
  if (fread(&n, sizeof(n), 1, f) != 1) std::exit(3);
  std::vector<T> v(n);
  if (n && fread(v.data(), sizeof(T), n, f) != (size_t)n) std::exit(3);
  return v;
}

int main(int argc, char** argv) {
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  auto dims = read_array<int64_t>(f);                 // n, R, P
  auto react = read_array<int64_t>(f);
  auto s_indptr = read_array<int32_t>(f), s_idx = read_array<int32_t>(f);
  auto s_val = read_array<double>(f);
  auto rows = read_array<int64_t>(f), cols = read_array<int64_t>(f);
  auto j_indptr = read_array<int32_t>(f), j_idx = read_array<int32_t>(f);
  auto j_val = read_array<double>(f);
  fclose(f);
  fo_mechanism_desc m = {(int32_t)dims[0], (int32_t)dims[1], (int32_t)dims[2], react.data(), s_indptr.data(),
                         s_idx.data(), s_val.data(), (int32_t)rows.size(), rows.data(), cols.data(),
                         j_indptr.data(), j_idx.data(), j_val.data(), nullptr};
  fo::HostTables t;
  std::string err = fo::build_tables(m, FO_ORDER_AUTO, &t);
  if (!err.empty() || t.ce_ptr.empty()) {
    printf("tables: %s\n", err.c_str());
    return 1;
  }
  // Both packed elimination streams must be hazard-free within each chunk
  // (the device reads a chunk's work-row values before running it): no slot is
  // updated twice in a chunk, and no multiplier reads a slot an earlier update
  // of its chunk wrote. Rows (pipelined) and passes (compact) start on chunks.
  auto hazard_free = [](const std::vector<uint32_t>& st, const std::vector<int32_t>& ptr, uint32_t special) {
    for (int32_t p : ptr)
      if (p % fo::kStreamChunk) return false;
    for (size_t c0 = 0; c0 < st.size(); c0 += fo::kStreamChunk) {
      std::vector<uint32_t> updated;
      for (size_t w = c0; w < c0 + fo::kStreamChunk && w < st.size(); ++w) {
        const uint32_t word = st[w], y = word & 0x7fffu;
        if (!(word & 0x8000u) && y >= special) continue;        // padding or reload
        for (uint32_t u : updated)
          if (u == y) return false;
        if (!(word & 0x8000u)) updated.push_back(y);
      }
    }
    return true;
  };
  std::vector<int32_t> el_starts(t.el_ptr.begin(), t.el_ptr.end());
  if (!t.elp.empty() && !hazard_free(t.elp, el_starts, 0x7fffu)) return 17;
  if (!hazard_free(t.cep, t.ce_ptr, fo::kReloadSlot)) return 18;
  const int n = t.n, nlu = (int)t.lu_col.size(), nj = (int)t.j_col.size();
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  std::vector<double> negj(nj);
  for (double& v : negj) v = U(rng);
  const double alpha = 8.0 * n;                         // diagonally dominant: pivots stay away from zero
  // plain row-by-row LU (the device's FO_VARIANT_PLAIN loop)
  std::vector<double> ref(nlu, 0.0), w(n, 0.0);
  for (int r = 0; r < n; ++r) {
    const int q0 = t.lu_row_ptr[r], q1 = t.lu_row_ptr[r + 1], dg = t.lu_diag[r];
    for (int q = q0; q < q1; ++q) w[t.lu_col[q]] = 0.0;
    for (int e = t.j_row_ptr[r]; e < t.j_row_ptr[r + 1]; ++e) w[t.j_col[e]] = negj[e];
    w[r] = w[r] + alpha * t.mass[r];
    for (int q = q0; q < dg; ++q) {
      const int k = t.lu_col[q];
      const double l = w[k] * ref[t.lu_diag[k]];
      ref[q] = l;
      for (int u = t.lu_diag[k] + 1; u < t.lu_row_ptr[k + 1]; ++u) w[t.lu_col[u]] = std::fma(-l, ref[u], w[t.lu_col[u]]);
    }
    ref[dg] = 1.0 / w[r];
    for (int q = dg + 1; q < q1; ++q) ref[q] = w[t.lu_col[q]];
  }
  // compact: two passes per row over half-row work rows
  std::vector<double> lu(nlu, 0.0);
  for (int r = 0; r < n; ++r) {
    const int q0 = t.lu_row_ptr[r], len = t.lu_row_ptr[r + 1] - q0, dslot = t.lu_diag[r] - q0;
    const int split = t.cs_split[r];
    for (int pass = 0; pass < 2; ++pass) {
      const int base = pass ? split : 0, cnt = pass ? len - split : split;
      if (cnt > t.cmax_half) return 10;
      std::vector<double> h(cnt, 0.0);
      const int e0 = pass ? t.cs_jsplit[r] : t.j_row_ptr[r], e1 = pass ? t.j_row_ptr[r + 1] : t.cs_jsplit[r];
      for (int e = e0; e < e1; ++e) {
        const int s = t.j_lu_pos[e] - q0 - base;
        if (s < 0 || s >= cnt) return 11;
        h[s] = negj[e];
      }
      if (dslot >= base && dslot < base + cnt) h[dslot - base] = h[dslot - base] + alpha * t.mass[r];
      double l = 0.0;
      for (int e = t.ce_ptr[2 * r + pass]; e < t.ce_ptr[2 * r + pass + 1]; ++e) {
        const uint32_t word = t.cep[e], pos = word >> 16, y = word & 0x7fffu;
        if (word & 0x8000u) {
          if ((int)y >= cnt) return 12;
          l = h[y] * lu[pos];
          lu[q0 + base + y] = l;
        } else if (y == fo::kReloadSlot) {
          l = lu[pos];
        } else if (y != 0x7fffu) {
          if ((int)y >= cnt || (int)pos >= nlu) return 13;
          h[y] = std::fma(-l, lu[pos], h[y]);
        }
      }
      if (dslot >= base && dslot < base + cnt) h[dslot - base] = 1.0 / h[dslot - base];
      for (int s = std::max(dslot - base, 0); s < cnt; ++s) lu[q0 + base + s] = h[s];
    }
  }
  for (int q = 0; q < nlu; ++q)
    if (lu[q] != ref[q]) {
      printf("factor mismatch at %d: %.17g vs %.17g\n", q, lu[q], ref[q]);
      return 4;
    }
  // solves: plain (the device's lu_solve) and split (four streams, halves)
  std::vector<double> b(n), x(n);
  for (double& v : b) v = U(rng);
  for (int i = 0; i < n; ++i) x[i] = b[i];
  for (int r = 0; r < n; ++r) {
    double acc = x[r];
    for (int q = t.lu_row_ptr[r]; q < t.lu_diag[r]; ++q) acc = std::fma(-ref[q], x[t.lu_col[q]], acc);
    x[r] = acc;
  }
  for (int r = n - 1; r >= 0; --r) {
    double acc = x[r];
    for (int q = t.lu_diag[r] + 1; q < t.lu_row_ptr[r + 1]; ++q) acc = std::fma(-ref[q], x[t.lu_col[q]], acc);
    x[r] = acc * ref[t.lu_diag[r]];
  }
  const int mh = t.csm;
  if (std::max(mh, n - mh) > std::max(t.cmax_half, std::max(mh, n - mh))) return 14;
  std::vector<double> vec = b, stage(std::max(mh, n - mh), 0.0);
  auto run = [&](const std::vector<int32_t>& st, bool backward) -> int {
    double acc = 0.0;
    for (size_t e = 0; e < st.size(); e += 2) {
      const int32_t xx = st[e], y = st[e + 1];
      if (y == fo::kNoop) continue;
      if (y >= 0) {
        const double v = (y & fo::kGlobalOperand) ? vec[y & ~fo::kGlobalOperand] : stage[y];
        if (!(y & fo::kGlobalOperand) && y >= (int)stage.size()) return 15;
        acc = std::fma(-lu[xx], v, acc);
      } else {
        const int rr = -1 - y;
        const double s = stage[rr] + acc;
        stage[rr] = backward ? s * lu[-1 - xx] : s;
        acc = 0.0;
      }
    }
    return 0;
  };
  int rc = 0;
  for (int i = 0; i < mh; ++i) stage[i] = vec[i];
  rc |= run(t.csf_a, false);
  for (int i = 0; i < mh; ++i) vec[i] = stage[i];
  for (int i = mh; i < n; ++i) stage[i - mh] = vec[i];
  rc |= run(t.csf_b, false);
  rc |= run(t.csb_b, true);
  for (int i = mh; i < n; ++i) vec[i] = stage[i - mh];
  for (int i = 0; i < mh; ++i) stage[i] = vec[i];
  rc |= run(t.csb_a, true);
  for (int i = 0; i < mh; ++i) vec[i] = stage[i];
  if (rc) return rc;
  double worst = 0.0;
  for (int i = 0; i < n; ++i) worst = std::max(worst, std::fabs(vec[i] - x[i]) / std::max(std::fabs(x[i]), 1e-300));
  printf("n %d nnz_lu %d max_half %d halves %d/%d solve rel diff %.3e\n", n, nlu, t.cmax_half, mh, n - mh, worst);
  return worst <= 1e-12 ? 0 : 5;
}
