// Device functions of the Rosenbrock integrator: the mechanism evaluations,
// the sparse LU and its solves, the stage loop, the error norm, the
// controller and the projection of one group over one interval
// (fastode/solvers.py:37-415, chem.py:86-102, linalg.py:15-81), shared by the
// forward kernels (integrator.cu) and the adjoint kernels (adjoint.cu).
// Each translation unit that includes this file gets its own copy.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>

#include <cmath>
#include <cstdint>

#include "device.cuh"
#include "fastode_gb300.h"

#ifdef FO_LINK_GENERATED
// The mechanism's generated factorization and solves (codegen.cpp), linked in
// per mechanism: `base` is this lane's item 0 of its scratch slot (32 lanes),
// `mech` the mechanism's index in the module (several mechanisms share one).
extern "C" __device__ void fo_gen_factor(double* base, double alpha, int mech);
extern "C" __device__ void fo_gen_solve(double* base, int mech);
extern "C" __device__ void fo_gen_solve_t(double* base, int mech);   // the adjoint's transposed solve
#endif

namespace fo {
// internal linkage: every translation unit that includes this file keeps its
// own copy of these device functions
namespace {


#define SCR(base, item) (base)[(int64_t)(item) * L + lane]
#define WROW(c) w[(c) * L + lane]

__device__ __forceinline__ double pymin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double pymax(double a, double b) { return (b > a) ? b : a; }
// numpy.maximum: NaN if either operand is NaN
__device__ __forceinline__ double npmax(double a, double b) {
  if (a != a) return a;
  if (b != b) return b;
  return (a > b) ? a : b;
}
// numpy.maximum(y, 0.0): keeps NaN, maps -0.0 to 0.0
__device__ __forceinline__ double clamp0(double y) { return (y <= 0.0) ? 0.0 : y; }

// fastode/solvers.py:46-51
__device__ __forceinline__ double quantize_step(double h, double interval) {
  if (h >= interval) return interval;
  double q = ceil(__dsub_rn(__ddiv_rn(interval, h), 1.0e-9));
  if (!(q >= 1.0)) q = 1.0;
  return __ddiv_rn(interval, q);
}

struct Lane {
  int lane;      // thread index in the block
  int L;         // lanes per block
  int64_t cell;  // global cell index (clamped into the group for idle lanes)
  bool active;   // this lane owns a real cell of the group
};

// Rates r_j = k_j * prod(x[react[j, :]]) (fastode/chem.py:86-87). The
// arrays are distinct scratch items, so the loads of several reactions can be
// in flight together.
__device__ void eval_rates(const SolveParams& p, const Lane& ln, const double* __restrict__ x,
                           double* __restrict__ r) {
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n, R = p.t.R, P = p.t.P;
  const double* __restrict__ kc = p.k + ln.cell * p.kcs;
#pragma unroll 4
  for (int j = 0; j < R; ++j) {
    double prod = 1.0;
    for (int q = 0; q < P; ++q) {
      int s = __ldg(p.t.react + j * P + q);
      if (s != n) prod = __dmul_rn(prod, SCR(x, s));
    }
    SCR(r, j) = __dmul_rn(__ldg(kc + (int64_t)j * p.krs), prod);
  }
}

// Forcing F = S r, species rows of the permuted stoichiometry
// (fastode/chem.py:89-90). Each row's rates are loaded eight at a time
// before they are summed in order, so their latencies overlap.
__device__ void eval_forcing(const SolveParams& p, const Lane& ln, const double* __restrict__ r,
                             double* __restrict__ f) {
  constexpr int kBatch = 8;
  const int L = ln.L, lane = ln.lane;
  for (int i = 0; i < p.t.n; ++i) {
    double acc = 0.0;
    const int q1 = __ldg(p.t.s_ptr + i + 1);
    int q = __ldg(p.t.s_ptr + i);
    for (; q + kBatch <= q1; q += kBatch) {
      double v[kBatch];
#pragma unroll
      for (int b = 0; b < kBatch; ++b) v[b] = SCR(r, __ldg(p.t.s_rxn + q + b));
#pragma unroll
      for (int b = 0; b < kBatch; ++b) acc = fma(__ldg(p.t.s_val + q + b), v[b], acc);
    }
    for (; q < q1; ++q) acc = fma(__ldg(p.t.s_val + q), SCR(r, __ldg(p.t.s_rxn + q)), acc);
    SCR(f, i) = acc;
  }
}

__device__ __noinline__ void eval_rhs(const SolveParams& p, const Lane& ln, const double* x, double* r, double* f) {
  eval_rates(p, ln, x, r);
  eval_forcing(p, ln, r, f);
}

// Negated Jacobian values in assembly order: d[j,p] = k_j prod_{q != p} x_q,
// then -J = sum of (-S[i,j]) d[j,p] over the map's terms
// (fastode/chem.py:92-102).
__device__ __noinline__ void eval_negjac(const SolveParams& p, const Lane& ln, const double* __restrict__ x,
                                         double* __restrict__ d, double* __restrict__ negj) {
  constexpr int kBatch = 8;
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n, R = p.t.R, P = p.t.P;
  const double* __restrict__ kc = p.k + ln.cell * p.kcs;
#pragma unroll 4
  for (int j = 0; j < R; ++j) {
    const double kj = __ldg(kc + (int64_t)j * p.krs);
    for (int a = 0; a < P; ++a) {
      double prod = kj;
      for (int q = 0; q < P; ++q) {
        if (q == a) continue;
        int s = __ldg(p.t.react + j * P + q);
        if (s != n) prod = __dmul_rn(prod, SCR(x, s));
      }
      SCR(d, j * P + a) = prod;
    }
  }
  for (int e = 0; e < p.t.nnzj; ++e) {
    double acc = 0.0;
    const int t1 = __ldg(p.t.jt_ptr + e + 1);
    int t = __ldg(p.t.jt_ptr + e);
    for (; t + kBatch <= t1; t += kBatch) {
      double v[kBatch];
#pragma unroll
      for (int b = 0; b < kBatch; ++b) v[b] = SCR(d, __ldg(p.t.jt_idx + t + b));
#pragma unroll
      for (int b = 0; b < kBatch; ++b) acc = __dadd_rn(acc, __dmul_rn(__ldg(p.t.jt_val + t + b), v[b]));
    }
    for (; t < t1; ++t) acc = __dadd_rn(acc, __dmul_rn(__ldg(p.t.jt_val + t), SCR(d, __ldg(p.t.jt_idx + t))));
    SCR(negj, e) = acc;
  }
}

// Row r of the stage matrix alpha*M - J scattered into the dense work row w
// over the row's filled pattern (fastode/linalg.py:60-67). With alg_only,
// the projection's matrix diag(M) - J with the differential rows of J
// dropped (fastode/linalg.py:62-63, alpha = 1).
__device__ __forceinline__ void assemble_row(const SolveParams& p, const Lane& ln, int r, int q0, int q1,
                                             double alpha, const double* negj, double* w, bool alg_only) {
  const int L = ln.L, lane = ln.lane;
  const int32_t* __restrict__ col = p.t.lu_col;
  for (int q = q0; q < q1; ++q) WROW(__ldg(col + q)) = 0.0;
  const double mr = __ldg(p.t.mass + r);
  if (!alg_only || mr == 0.0) {
    const int e1 = __ldg(p.t.j_row_ptr + r + 1);
    for (int e = __ldg(p.t.j_row_ptr + r); e < e1; ++e) WROW(__ldg(p.t.j_col + e)) = SCR(negj, e);
  }
  WROW(r) = __dadd_rn(WROW(r), __dmul_rn(alpha, mr));
}

// In-place pivot-free LU of alpha*M - J on the precomputed fill pattern,
// row by row (up-looking). Row r is scattered into the dense work row w,
// eliminated with the finished rows above it, and gathered back. The
// diagonal slot keeps the reciprocal of the pivot. Replaces SuperLU's gstrf
// (fastode/linalg.py:70-78) and LAPACK getrf (fastode/linalg.py:15-18).
__device__ __noinline__ void factor(const SolveParams& p, const Lane& ln, double alpha, const double* negj, double* lu,
                       double* w, bool alg_only) {
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n;
  const int32_t* __restrict__ rowp = p.t.lu_row_ptr;
  const int32_t* __restrict__ diag = p.t.lu_diag;
  const int32_t* __restrict__ col = p.t.lu_col;
  for (int r = 0; r < n; ++r) {
    const int q0 = __ldg(rowp + r), q1 = __ldg(rowp + r + 1), dg = __ldg(diag + r);
    assemble_row(p, ln, r, q0, q1, alpha, negj, w, alg_only);
    for (int q = q0; q < dg; ++q) {
      const int k = __ldg(col + q);
      const double l = WROW(k) * SCR(lu, __ldg(diag + k));
      SCR(lu, q) = l;
      const int u1 = __ldg(rowp + k + 1);
      int u = __ldg(diag + k) + 1;
      for (; u + 3 < u1; u += 4) {
        const int c0 = __ldg(col + u), c1 = __ldg(col + u + 1), c2 = __ldg(col + u + 2), c3 = __ldg(col + u + 3);
        const double v0 = SCR(lu, u), v1 = SCR(lu, u + 1), v2 = SCR(lu, u + 2), v3 = SCR(lu, u + 3);
        WROW(c0) = fma(-l, v0, WROW(c0));
        WROW(c1) = fma(-l, v1, WROW(c1));
        WROW(c2) = fma(-l, v2, WROW(c2));
        WROW(c3) = fma(-l, v3, WROW(c3));
      }
      for (; u < u1; ++u) {
        const int c = __ldg(col + u);
        WROW(c) = fma(-l, SCR(lu, u), WROW(c));
      }
    }
    SCR(lu, dg) = 1.0 / WROW(r);
    for (int q = dg + 1; q < q1; ++q) SCR(lu, q) = WROW(__ldg(col + q));
  }
}

// The same factorization driven by the precomputed elimination stream
// (symbolic.h): every row's multipliers and updates are one flat sequence of
// (x, y) entries in chunks of kChunk. The work row is compressed to the row's
// own pattern (w[y] stands for lu[row start + y]), which leaves room in shared
// memory for a ring of kRingChunks chunks: each lane copies its own 8-byte U
// entries (of finished rows, or pivot reciprocals — nothing the row writes)
// into the ring with cp.async several chunks ahead of their use, so a warp
// keeps up to (kRingChunks - 1) * kChunk 256-byte loads in flight without
// holding them in registers.
constexpr int kChunk = kStreamChunk;

// Stream metadata, packed to 32 bits per entry: (position << 16) | slot, slot
// bit 15 marking a multiplier, slot 0x7fff padding. A chunk is four uint4.
struct Meta {
  uint4 q[kChunk / 4];
};

__device__ __forceinline__ void meta_load(const uint32_t* __restrict__ m, Meta& out) {
#pragma unroll
  for (int i = 0; i < kChunk / 4; ++i) out.q[i] = __ldg(reinterpret_cast<const uint4*>(m) + i);
}

__device__ __forceinline__ uint32_t meta_at(const Meta& m, int s) {
  const uint4 v = m.q[s >> 2];
  return (s & 3) == 0 ? v.x : (s & 3) == 1 ? v.y : (s & 3) == 2 ? v.z : v.w;
}

// Copy the chunk's 16 operands of this lane (U entries of finished rows or
// pivot reciprocals; padding copies entry 0) into the ring slot.
__device__ __forceinline__ void ring_issue(const Meta& m, const double* __restrict__ lu, int L, int lane,
                                           double* ring_slot) {
  const unsigned dst0 = (unsigned)__cvta_generic_to_shared(ring_slot + lane);
#pragma unroll
  for (int s = 0; s < kChunk; ++s) {
    const uint32_t word = meta_at(m, s);
    const double* g = lu + (int64_t)(word >> 16) * L + lane;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst0 + (unsigned)(s * L * 8)), "l"(g));
  }
}

__device__ __forceinline__ void ring_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

__device__ __forceinline__ void ring_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(kRingChunks - 1) : "memory");
}

// A hazard-free chunk (symbolic.cpp builds them) in three parts: read every
// work-row value the chunk touches, apply its multipliers and updates in order
// in registers (updates are independent FMAs; only a multiplier starts a new
// dependency), and write the updated values back. The factorization writes a
// chunk back only after the next chunk has read its values and issued its
// FMAs, which the two-chunk hazard rule makes safe.
__device__ __forceinline__ void chunk_read(const Meta& m, const double* w, int L, int lane, double (&wv)[kChunk]) {
#pragma unroll
  for (int s = 0; s < kChunk; ++s) {
    const uint32_t y = meta_at(m, s) & 0x7fffu;
    wv[s] = y != 0x7fffu ? WROW(y) : 0.0;
  }
}

__device__ __forceinline__ void chunk_fma(const Meta& m, const double* ring_slot, double* lu, int L, int lane,
                                          double (&wv)[kChunk], double& l, int& q) {
#pragma unroll
  for (int s = 0; s < kChunk; ++s) {
    const uint32_t word = meta_at(m, s);
    const uint32_t y = word & 0x7fffu;
    const double v = ring_slot[s * L + lane];
    if (word & 0x8000u) {
      l = wv[s] * v;
      SCR(lu, q) = l;
      ++q;
    } else if (y != 0x7fffu) {
      wv[s] = fma(-l, v, wv[s]);
    }
  }
}

__device__ __forceinline__ void chunk_write(const Meta& m, double* w, int L, int lane, const double (&wv)[kChunk]) {
#pragma unroll
  for (int s = 0; s < kChunk; ++s) {
    const uint32_t word = meta_at(m, s);
    const uint32_t y = word & 0x7fffu;
    if (!(word & 0x8000u) && y != 0x7fffu) WROW(y) = wv[s];
  }
}

template <int kL>
__device__ __noinline__ void factor_stream(const SolveParams& p, const Lane& ln, double alpha, const double* negj,
                                           double* lu, double* w, bool alg_only) {
  const int L = kL ? kL : ln.L, lane = ln.lane;
  const int n = p.t.n;
  const int32_t* __restrict__ rowp = p.t.lu_row_ptr;
  const int32_t* __restrict__ diag = p.t.lu_diag;
  double* ring = w + (int64_t)p.t.max_row_len * L;
  for (int r = 0; r < n; ++r) {
    const int q0 = __ldg(rowp + r), q1 = __ldg(rowp + r + 1), dg = __ldg(diag + r);
    // assemble row r of alpha*M - J into the compressed work row
    for (int s = 0; s < q1 - q0; ++s) WROW(s) = 0.0;
    const double mr = __ldg(p.t.mass + r);
    if (!alg_only || mr == 0.0) {
      const int e1 = __ldg(p.t.j_row_ptr + r + 1);
      for (int e = __ldg(p.t.j_row_ptr + r); e < e1; ++e) WROW(__ldg(p.t.j_pos + e) - q0) = SCR(negj, e);
    }
    WROW(dg - q0) = __dadd_rn(WROW(dg - q0), __dmul_rn(alpha, mr));
    const int t0 = __ldg(p.t.el_ptr + r);
    const int nch = (__ldg(p.t.el_ptr + r + 1) - t0) / kChunk;
    const uint32_t* meta = p.t.elp + t0;
    double l = 0.0;
    int q = q0;
    Meta mi, mc;
#pragma unroll 1
    for (int c = 0; c < kRingChunks - 1; ++c) {
      if (c < nch) {
        meta_load(meta + c * kChunk, mi);
        ring_issue(mi, lu, L, lane, ring + (int64_t)(c % kRingChunks) * kChunk * L);
      }
      ring_commit();
    }
    if (kRingChunks - 1 < nch) meta_load(meta + (kRingChunks - 1) * kChunk, mi);
    if (nch > 0) meta_load(meta, mc);
#pragma unroll 1
    for (int c = 0; c < nch; ++c) {
      const int ahead = c + kRingChunks - 1;
      Meta mi_next, mc_next;
      if (ahead + 1 < nch) meta_load(meta + (ahead + 1) * kChunk, mi_next);
      if (c + 1 < nch) meta_load(meta + (c + 1) * kChunk, mc_next);
      if (ahead < nch) ring_issue(mi, lu, L, lane, ring + (int64_t)(ahead % kRingChunks) * kChunk * L);
      ring_commit();
      ring_wait();
      double wc[kChunk];
      chunk_read(mc, w, L, lane, wc);
      chunk_fma(mc, ring + (int64_t)(c % kRingChunks) * kChunk * L, lu, L, lane, wc, l, q);
      chunk_write(mc, w, L, lane, wc);
      mi = mi_next;
      mc = mc_next;
    }
    SCR(lu, dg) = 1.0 / WROW(dg - q0);
    for (int qq = dg + 1; qq < q1; ++qq) SCR(lu, qq) = WROW(qq - q0);
  }
}

// ---- the compact factorization (FO_VARIANT_COMPACT) ------------------------------
//
// Row r is eliminated in two passes over halves of its slots (symbolic.h):
// pass A is the elimination restricted to the row's leading columns and
// stores its multipliers as it makes them; pass B applies every multiplier's
// updates of the trailing columns, in the same order, reloading A's
// multipliers from the LU storage through the same ring as the U operands (a
// block-scope fence between the passes orders this thread's stores of them
// before the asynchronous copies that read them back). The work row therefore
// holds half a row, and the factors are the pipelined ones bit for bit. The
// operands are staged one chunk ahead in a two-slot ring: with twice as many
// groups resident per SM, a deeper ring buys nothing.

template <int kL>
__device__ __noinline__ void factor_compact(const SolveParams& p, const Lane& ln, double alpha, const double* negj,
                                            double* lu, double* w, bool alg_only) {
  const int L = kL ? kL : ln.L, lane = ln.lane;
  const int n = p.t.n;
  const int32_t* __restrict__ rowp = p.t.lu_row_ptr;
  const int32_t* __restrict__ diag = p.t.lu_diag;
  double* ring = w + (int64_t)p.t.cmax_half * L;
  for (int r = 0; r < n; ++r) {
    const int q0 = __ldg(rowp + r), len = __ldg(rowp + r + 1) - q0, dslot = __ldg(diag + r) - q0;
    const int split = __ldg(p.t.cs_split + r), jsplit = __ldg(p.t.cs_jsplit + r);
    const double mr = __ldg(p.t.mass + r);
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
      const int base = pass ? split : 0, cnt = pass ? len - split : split;
      for (int s = 0; s < cnt; ++s) WROW(s) = 0.0;
      if (!alg_only || mr == 0.0) {
        const int e0 = pass ? jsplit : __ldg(p.t.j_row_ptr + r);
        const int e1 = pass ? __ldg(p.t.j_row_ptr + r + 1) : jsplit;
        for (int e = e0; e < e1; ++e) WROW(__ldg(p.t.j_pos + e) - q0 - base) = SCR(negj, e);
      }
      const bool has_diag = dslot >= base && dslot < base + cnt;
      if (has_diag) WROW(dslot - base) = __dadd_rn(WROW(dslot - base), __dmul_rn(alpha, mr));
      const int t0 = __ldg(p.t.ce_ptr + 2 * r + pass);
      const int nch = (__ldg(p.t.ce_ptr + 2 * r + pass + 1) - t0) / kChunk;
      const uint32_t* meta = p.t.cep + t0;
      double* qlu = lu + (int64_t)(q0 + base) * L;     // this pass's slot s stands for lu[q0 + base + s]
      double l = 0.0;
      Meta mc, mi;
      if (pass) __threadfence_block();   // pass A's stores before pass B's copies read them
      if (nch > 0) {
        meta_load(meta, mc);
        ring_issue(mc, lu, L, lane, ring);
      }
      ring_commit();
      if (nch > 1) meta_load(meta + kChunk, mi);
#pragma unroll 1
      for (int c = 0; c < nch; ++c) {
        Meta mn;
        if (c + 2 < nch) meta_load(meta + (c + 2) * kChunk, mn);
        if (c + 1 < nch) ring_issue(mi, lu, L, lane, ring + (int64_t)((c + 1) % kCompactRing) * kChunk * L);
        ring_commit();
        asm volatile("cp.async.wait_group %0;" ::"n"(kCompactRing - 1) : "memory");
        const double* rs = ring + (int64_t)(c % kCompactRing) * kChunk * L;
        double wv[kChunk];
#pragma unroll
        for (int s = 0; s < kChunk; ++s) {
          const uint32_t y = meta_at(mc, s) & 0x7fffu;
          wv[s] = y < kReloadSlot ? WROW(y) : 0.0;
        }
#pragma unroll
        for (int s = 0; s < kChunk; ++s) {
          const uint32_t word = meta_at(mc, s);
          const uint32_t y = word & 0x7fffu;
          if (word & 0x8000u) {
            l = wv[s] * rs[s * L + lane];
            SCR(qlu, y) = l;
          } else if (y == kReloadSlot) {
            l = rs[s * L + lane];
          } else if (y != 0x7fffu) {
            wv[s] = fma(-l, rs[s * L + lane], wv[s]);
          }
        }
#pragma unroll
        for (int s = 0; s < kChunk; ++s) {
          const uint32_t word = meta_at(mc, s);
          const uint32_t y = word & 0x7fffu;
          if (!(word & 0x8000u) && y < kReloadSlot) WROW(y) = wv[s];
        }
        mc = mi;
        mi = mn;
      }
      if (has_diag) WROW(dslot - base) = 1.0 / WROW(dslot - base);
      for (int s = dslot > base ? dslot - base : 0; s < cnt; ++s) SCR(qlu, s) = WROW(s);
    }
  }
}

// Forward and backward substitution driven by the solve streams
// (symbolic.h): a chunk's metadata is loaded two chunks ahead of its use and
// its factor entries one chunk ahead (neither depends on the solution), so the
// entries' loads never wait for their positions; the solution entries are read
// from shared memory when the chunk computes. kMixed: an operand may lie in
// the other, finished half of the vector in global memory (kGlobalOperand).
template <bool kMixed>
__device__ __forceinline__ void solve_values(const int4 (&m)[kChunk / 2], const double* __restrict__ lu,
                                             const double* xg, int L, int lane, double (&v)[kChunk],
                                             double (&g)[kChunk]) {
#pragma unroll
  for (int s = 0; s < kChunk / 2; ++s) {
    const int p0 = m[s].x >= 0 ? m[s].x : -1 - m[s].x;
    const int p1 = m[s].z >= 0 ? m[s].z : -1 - m[s].z;
    v[2 * s] = lu[(int64_t)p0 * L + lane];
    v[2 * s + 1] = lu[(int64_t)p1 * L + lane];
    if (kMixed) {
      const int y0 = m[s].y, y1 = m[s].w;
      g[2 * s] = (y0 >= 0 && (y0 & kGlobalOperand)) ? xg[(int64_t)(y0 & ~kGlobalOperand) * L + lane] : 0.0;
      g[2 * s + 1] = (y1 >= 0 && (y1 & kGlobalOperand)) ? xg[(int64_t)(y1 & ~kGlobalOperand) * L + lane] : 0.0;
    }
  }
}

__device__ __forceinline__ void solve_meta(const int2* __restrict__ meta, int4 (&m)[kChunk / 2]) {
#pragma unroll
  for (int s = 0; s < kChunk / 2; ++s) m[s] = __ldg(reinterpret_cast<const int4*>(meta) + s);
}

// Two partial sums per row, entry s of a chunk feeding sum s mod 2: the row's
// FMAs form two independent chains. More sums hide more FP64 latency but cost
// registers the chunk buffers need (measured per interval: four sums 4.5%
// slower, eight 10% slower).
template <bool kBackward, bool kMixed>
__device__ __forceinline__ void solve_entry(int s, int y, double v, double gv, double* w, int L, int lane,
                                            double (&acc)[2]) {
  if (y >= 0) {
    const double x = (kMixed && (y & kGlobalOperand)) ? gv : WROW(y);
    acc[s & 1] = fma(-v, x, acc[s & 1]);
  } else if (y != kNoop) {
    const int r = -1 - y;
    const double b = WROW(r) + (acc[0] + acc[1]);
    WROW(r) = kBackward ? b * v : b;
    acc[0] = acc[1] = 0.0;
  }
}

template <bool kBackward, bool kMixed>
__device__ __forceinline__ void solve_compute(const int4 (&m)[kChunk / 2], const double (&v)[kChunk],
                                              const double (&g)[kChunk], double* w, int L, int lane, double (&acc)[2]) {
#pragma unroll
  for (int s = 0; s < kChunk / 2; ++s) {
    solve_entry<kBackward, kMixed>(2 * s, m[s].y, v[2 * s], g[2 * s], w, L, lane, acc);
    solve_entry<kBackward, kMixed>(2 * s + 1, m[s].w, v[2 * s + 1], g[2 * s + 1], w, L, lane, acc);
  }
}

// kMixed: the stream's operands may lie in xg (kGlobalOperand set).
template <bool kBackward, bool kMixed = false>
__device__ __forceinline__ void solve_stream(const int2* __restrict__ st, int nst, const double* lu, double* w, int L,
                                             int lane,
                             const double* xg = nullptr) {
  int4 mc[kChunk / 2], mn[kChunk / 2];
  double vc[kChunk], gc[kChunk];
  double acc[2] = {0.0, 0.0};
  const int nch = nst / kChunk;
  if (nch == 0) return;            // an empty half (a one-species system)
  solve_meta(st, mc);
  solve_values<kMixed>(mc, lu, xg, L, lane, vc, gc);
  if (nch > 1) solve_meta(st + kChunk, mn);
#pragma unroll 1
  for (int c = 0; c < nch; ++c) {
    int4 mnn[kChunk / 2];
    double vn[kChunk], gn[kChunk];
    if (c + 1 < nch) solve_values<kMixed>(mn, lu, xg, L, lane, vn, gn);
    if (c + 2 < nch) solve_meta(st + (c + 2) * kChunk, mnn);
    solve_compute<kBackward, kMixed>(mc, vc, gc, w, L, lane, acc);
#pragma unroll
    for (int s = 0; s < kChunk / 2; ++s) {
      mc[s] = mn[s];
      mn[s] = mnn[s];
    }
#pragma unroll
    for (int s = 0; s < kChunk; ++s) {
      vc[s] = vn[s];
      gc[s] = gn[s];
    }
  }
}

template <int kL>
__device__ __noinline__ void lu_solve_pipelined(const SolveParams& p, const Lane& ln, const double* lu, double* w) {
  const int L = kL ? kL : ln.L;
  solve_stream<false>(p.t.sf, p.t.nsf, lu, w, L, ln.lane);
  solve_stream<true>(p.t.sb, p.t.nsb, lu, w, L, ln.lane);
}

// The compact solves: b and x are per-lane vectors in global memory (they may
// alias) and shared memory holds one half of the vector at a time. Forward
// over rows [0, csm) needs only that half; the finished half is stored, and
// forward over rows [csm, n) then reads it from x, as does nothing else until
// backward over rows [n-1, csm) has finished the second half, which is stored
// for backward over rows [csm-1, 0) to read.
template <int kL>
__device__ __noinline__ void lu_solve_compact_l(const SolveParams& p, const Lane& ln, const double* lu, double* w,
                                                const double* b, double* x) {
  const int L = kL ? kL : ln.L, lane = ln.lane;
  const int n = p.t.n, m = p.t.csm;
  for (int i = 0; i < m; ++i) WROW(i) = SCR(b, i);
  solve_stream<false>(p.t.csf_a, p.t.ncsf_a, lu, w, L, lane);
  for (int i = 0; i < m; ++i) SCR(x, i) = WROW(i);
  for (int i = m; i < n; ++i) WROW(i - m) = SCR(b, i);
  solve_stream<false, true>(p.t.csf_b, p.t.ncsf_b, lu, w, L, lane, x);
  solve_stream<true>(p.t.csb_b, p.t.ncsb_b, lu, w, L, lane);
  for (int i = m; i < n; ++i) SCR(x, i) = WROW(i - m);
  for (int i = 0; i < m; ++i) WROW(i) = SCR(x, i);
  solve_stream<true, true>(p.t.csb_a, p.t.ncsb_a, lu, w, L, lane, x);
  for (int i = 0; i < m; ++i) SCR(x, i) = WROW(i);
}

// The stream kernels specialised for 32 lanes (one warp per group, the usual
// launch) fold the lane stride into immediate offsets; other group sizes run
// the general instantiation.
__device__ __forceinline__ void lu_solve_compact(const SolveParams& p, const Lane& ln, const double* lu, double* w,
                                                 const double* b, double* x) {
  if (ln.L == 32) lu_solve_compact_l<32>(p, ln, lu, w, b, x);
  else lu_solve_compact_l<0>(p, ln, lu, w, b, x);
}

// Forward and backward substitution in place on w (fastode/linalg.py:80-81).
__device__ void lu_solve(const SolveParams& p, const Lane& ln, const double* lu, double* w) {
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n;
  const int32_t* __restrict__ rowp = p.t.lu_row_ptr;
  const int32_t* __restrict__ diag = p.t.lu_diag;
  const int32_t* __restrict__ col = p.t.lu_col;
  for (int r = 0; r < n; ++r) {
    double acc = WROW(r);
    const int dg = __ldg(diag + r);
    for (int q = __ldg(rowp + r); q < dg; ++q) acc = fma(-SCR(lu, q), WROW(__ldg(col + q)), acc);
    WROW(r) = acc;
  }
  for (int r = n - 1; r >= 0; --r) {
    double acc = WROW(r);
    const int dg = __ldg(diag + r), q1 = __ldg(rowp + r + 1);
    for (int q = dg + 1; q < q1; ++q) acc = fma(-SCR(lu, q), WROW(__ldg(col + q)), acc);
    WROW(r) = acc * SCR(lu, dg);
  }
}

// The generated variant (FO_VARIANT_GENERATED) exists only in the kernels
// linked per mechanism with the generated functions.
// Those kernels run nothing else (the launch code guarantees the variant),
// so the other variants' factorizations and solves are not compiled into
// them.
__device__ __forceinline__ bool generated(const SolveParams&) {
#ifdef FO_LINK_GENERATED
  return true;
#else
  return false;
#endif
}

// The variants that solve a per-lane vector in place rather than the work row.
__device__ __forceinline__ bool solves_in_place(const SolveParams& p) {
  return p.o.variant == FO_VARIANT_COMPACT || generated(p);
}

__device__ void factor_any(const SolveParams& p, const Lane& ln, double alpha, const double* negj, double* lu,
                           double* w, bool alg_only) {
#ifdef FO_LINK_GENERATED
  // the projection's algebraic-rows-only matrix takes the row loop (the same
  // factors, in the same storage, bit for bit)
  if (alg_only) factor(p, ln, alpha, negj, lu, w, alg_only);
  else fo_gen_factor(lu - p.sl.lu * ln.L + ln.lane, alpha, p.o.gen_index);
#else
  if (p.o.variant == FO_VARIANT_PLAIN) factor(p, ln, alpha, negj, lu, w, alg_only);
  else if (p.o.variant == FO_VARIANT_COMPACT) {
    if (ln.L == 32) factor_compact<32>(p, ln, alpha, negj, lu, w, alg_only);
    else factor_compact<0>(p, ln, alpha, negj, lu, w, alg_only);
  } else {
    if (ln.L == 32) factor_stream<32>(p, ln, alpha, negj, lu, w, alg_only);
    else factor_stream<0>(p, ln, alpha, negj, lu, w, alg_only);
  }
#endif
}

__device__ __forceinline__ void solve_in_w(const SolveParams& p, const Lane& ln, const double* lu, double* w) {
  if (p.o.variant == FO_VARIANT_PLAIN) lu_solve(p, ln, lu, w);
  else if (ln.L == 32) lu_solve_pipelined<32>(p, ln, lu, w);
  else lu_solve_pipelined<0>(p, ln, lu, w);
}

// x = A^-1 b with the factors in lu (b and x per-lane vectors, may alias).
__device__ void solve_into(const SolveParams& p, const Lane& ln, const double* lu, double* w, const double* b,
                           double* x) {
#ifdef FO_LINK_GENERATED
  // the generated solves work on the slot's solve vector (item xs), whose
  // offset they know, so every access is an immediate offset from one base
  const int L = ln.L, lane = ln.lane;
  double* base = const_cast<double*>(lu) - p.sl.lu * L;
  double* xs = base + p.sl.xs * L;
  for (int i = 0; i < p.t.n; ++i) SCR(xs, i) = SCR(b, i);
  fo_gen_solve(base + lane, p.o.gen_index);
  for (int i = 0; i < p.t.n; ++i) SCR(x, i) = SCR(xs, i);
#else
  if (p.o.variant == FO_VARIANT_COMPACT) {
    lu_solve_compact(p, ln, lu, w, b, x);
    return;
  }
  const int L = ln.L, lane = ln.lane;
  for (int i = 0; i < p.t.n; ++i) WROW(i) = SCR(b, i);
  solve_in_w(p, ln, lu, w);
  for (int i = 0; i < p.t.n; ++i) SCR(x, i) = WROW(i);
#endif
}

// Sum over the block of one value per thread; every thread gets the same
// bits (xor butterfly, then the warp totals in warp order).
__device__ double block_sum(double v, double* red) {
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  const int nw = blockDim.x >> 5;
  if (nw == 1) return v;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = red[0];
  for (int i = 1; i < nw; ++i) s += red[i];
  return s;
}

// One attempt's stages (fastode/solvers.py:54-86), then Y_new, the error
// estimate and this lane's share of the error norm (fastode/solvers.py:37-43).
__device__ __noinline__ double attempt(const SolveParams& p, const Lane& ln, double H, const double* Y, double* Ynew,
                                       double* scr, double* w, long long& c_rhs, long long& c_solves,
                                       double* U = nullptr) {
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n;
  const DevTableau& tb = p.o.tab;
  const bool dae = p.t.has_constraints != 0;
  double* F0 = scr + p.sl.f0 * L;
  double* Ft = scr + p.sl.ft * L;
  double* Yr = scr + p.sl.yr * L;
  double* K = scr + p.sl.k * L;
  double* lu = scr + p.sl.lu * L;
  double* rr = scr + p.sl.r * L;
  const double* forcing = F0;
  for (int r = 0; r < tb.S; ++r) {
    if (r > 0 && tb.new_forcing[r]) {
      for (int i = 0; i < n; ++i) {
        double v = SCR(Y, i);
        for (int s = 0; s < r; ++s)
          if (tb.a[r][s] != 0.0) v = __dadd_rn(v, __dmul_rn(tb.a[r][s], SCR(K + (int64_t)s * n * L, i)));
        SCR(Yr, i) = v;
        if (U != nullptr) SCR(U + (int64_t)r * n * L, i) = v;   // stage point kept for the adjoint
      }
      eval_rhs(p, ln, Yr, rr, Ft);
      ++c_rhs;
      forcing = Ft;
    }
    double* Kr = K + (int64_t)r * n * L;
    const bool in_place = solves_in_place(p);   // right-hand side in Kr, solved in place
    // the stage's c(r, s) / H once per stage rather than once per species
    // (the same quotients, so the same sums bit for bit)
    double coefs[4];
    for (int s = 0; s < r; ++s) coefs[s] = __ddiv_rn(tb.c[r][s], H);
    for (int i = 0; i < n; ++i) {
      double v = SCR(forcing, i);
      for (int s = 0; s < r; ++s) {
        const double coef = coefs[s];
        if (coef != 0.0) {
          double ks = SCR(K + (int64_t)s * n * L, i);
          if (dae) ks = __dmul_rn(ks, __ldg(p.t.mass + i));
          v = __dadd_rn(v, __dmul_rn(coef, ks));
        }
      }
      if (in_place) SCR(Kr, i) = v;
      else WROW(i) = v;
    }
    if (in_place) {
      solve_into(p, ln, lu, w, Kr, Kr);
    } else {
      solve_in_w(p, ln, lu, w);
      for (int i = 0; i < n; ++i) SCR(Kr, i) = WROW(i);
    }
    ++c_solves;
  }
  // Y_new, E and the weighted sum of squares
  double acc = 0.0;
  for (int i = 0; i < n; ++i) {
    const double y = SCR(Y, i);
    double yn = y, e = 0.0;
    for (int r = 0; r < tb.S; ++r) {
      const double kv = SCR(K + (int64_t)r * n * L, i);
      if (tb.m[r] != 0.0) yn = __dadd_rn(yn, __dmul_rn(tb.m[r], kv));
      if (tb.e[r] != 0.0) e = __dadd_rn(e, __dmul_rn(tb.e[r], kv));
    }
    SCR(Ynew, i) = yn;
    // the restarting loop replaces the algebraic rows of the estimate by the
    // step change (fastode/solvers.py:238-239)
    if (p.o.loop == FO_LOOP_RESTARTING && p.o.step_change_rows && dae && __ldg(p.t.mass + i) == 0.0)
      e = __dsub_rn(yn, y);
    const double ymax = npmax(fabs(y), fabs(yn));
    const double s = __ddiv_rn(e, __dadd_rn(__ldg(p.atol + __ldg(p.t.perm + i)), __dmul_rn(p.rtol, ymax)));
    acc = __dadd_rn(acc, __dmul_rn(s, s));
  }
  return ln.active ? acc : 0.0;
}

__device__ void trace_record(const SolveParams& p, int g, int& nrec, double t, double H, double err, double outcome) {
  if (p.trace == nullptr || threadIdx.x != 0) {
    ++nrec;
    return;
  }
  if (nrec < p.trace_cap) {
    double* rec = p.trace + ((int64_t)g * p.trace_cap + nrec) * 4;
    rec[0] = t;
    rec[1] = H;
    rec[2] = err;
    rec[3] = outcome;
  }
  ++nrec;
}

// Block-wide max with NaN propagation (numpy max) and block-wide AND.
__device__ double block_max(double v, double* red) {
  for (int off = 16; off > 0; off >>= 1) v = npmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  const int nw = blockDim.x >> 5;
  if (nw == 1) return v;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = red[0];
  for (int i = 1; i < nw; ++i) s = npmax(s, red[i]);
  return s;
}

__device__ bool block_all(bool v) {
  return __syncthreads_and(v ? 1 : 0) != 0;
}

struct ProjectionCounts {
  long long rhs = 0, jac = 0, lu = 0, solves = 0, passes = 0, trials = 0;
};

// All algebraic entries of A (a per-lane vector) finite, over the group.
__device__ bool alg_finite(const SolveParams& p, const Lane& ln, const double* A) {
  const int L = ln.L, lane = ln.lane;
  bool ok = true;
  if (ln.active)
    for (int i = 0; i < p.t.n; ++i)
      if (__ldg(p.t.mass + i) == 0.0 && !isfinite(SCR(A, i))) ok = false;
  return block_all(ok);
}

// max over the group's algebraic entries of |A|
__device__ double alg_absmax(const SolveParams& p, const Lane& ln, const double* A, double* red) {
  const int L = ln.L, lane = ln.lane;
  double m = 0.0;
  if (ln.active)
    for (int i = 0; i < p.t.n; ++i)
      if (__ldg(p.t.mass + i) == 0.0) m = npmax(m, fabs(SCR(A, i)));
  return block_max(m, red);
}

// The weighted Newton correction of fastode/solvers.py:119-124:
// max over algebraic entries of |d| / (atol + rtol max(|z|, |z + d|)), with
// 0 where d = 0 and the scale vanishes, inf where only the scale vanishes.
__device__ double weighted(const SolveParams& p, const Lane& ln, const double* Z, const double* D, double* red) {
  const int L = ln.L, lane = ln.lane;
  double m = 0.0;
  if (ln.active)
    for (int i = 0; i < p.t.n; ++i) {
      if (__ldg(p.t.mass + i) != 0.0) continue;
      const double z = SCR(Z, i), d = SCR(D, i);
      const double scale =
          __dadd_rn(__ldg(p.atol + __ldg(p.t.perm + i)), __dmul_rn(p.rtol, npmax(fabs(z), fabs(__dadd_rn(z, d)))));
      double q;
      if (scale > 0.0) q = __ddiv_rn(fabs(d), scale);
      else if (scale != scale) q = scale;
      else q = (d == 0.0) ? 0.0 : CUDART_INF;
      m = npmax(m, q);
    }
  return block_max(m, red);
}

// G = F(Z) with the differential rows zeroed (fastode/solvers.py:110-114).
__device__ void alg_residual(const SolveParams& p, const Lane& ln, const double* Z, double* rr, double* G) {
  const int L = ln.L, lane = ln.lane;
  eval_rhs(p, ln, Z, rr, G);
  for (int i = 0; i < p.t.n; ++i)
    if (__ldg(p.t.mass + i) != 0.0) SCR(G, i) = 0.0;
}

__device__ void factor_any(const SolveParams& p, const Lane& ln, double alpha, const double* negj, double* lu,
                           double* w, bool alg_only);
__device__ void solve_into(const SolveParams& p, const Lane& ln, const double* lu, double* w, const double* b,
                           double* x);

// Consistent initialization of the algebraic species, fastode/solvers.py:100-178:
// damped Newton with the algebraic-rows-only matrix (alpha = 1), accepted on
// the weighted correction, with backtracking line search. Returns true on
// convergence; on failure Y is restored to its value on entry.
// Every accepted update (Y += step * delta on the algebraic rows) is traced
// as (0, step, q, 2), so that the adjoint can replay the same updates.
__device__ __noinline__ bool project(const SolveParams& p, const Lane& ln, double* Y, double* scr, double* w, double* red,
                        ProjectionCounts& pc, int g, int& nrec) {
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n;
  double* G = scr + p.sl.f0 * L;
  double* cand = scr + p.sl.yr * L;
  double* orig = scr + p.sl.ynew * L;
  double* delta = scr + p.sl.k * L;
  double* trial = scr + (p.sl.k + n) * L;
  double* Gc = scr + p.sl.ft * L;
  double* rr = scr + p.sl.r * L;
  double* negj = scr + p.sl.negj * L;
  double* dd = scr + p.sl.d * L;
  double* lu = scr + p.sl.lu * L;
  const int max_updates = 10, max_backtracks = 24;
  const double tol = 0.1, factor_bt = 0.5, sigma = 1.0e-4;
  bool have_orig = false;
  for (int update = 0; update <= max_updates; ++update) {
    alg_residual(p, ln, Y, rr, G);
    ++pc.rhs;
    if (!alg_finite(p, ln, G)) break;
    ++pc.passes;
    if (alg_absmax(p, ln, G, red) == 0.0) return true;
    eval_negjac(p, ln, Y, dd, negj);
    ++pc.jac;
    factor_any(p, ln, 1.0, negj, lu, w, true);
    ++pc.lu;
    solve_into(p, ln, lu, w, G, delta);
    ++pc.solves;
    if (!alg_finite(p, ln, delta)) break;
    const double q = weighted(p, ln, Y, delta, red);
    if (q <= tol) return true;
    if (update == max_updates) break;
    if (!have_orig) {
      for (int i = 0; i < n; ++i) SCR(orig, i) = SCR(Y, i);
      have_orig = true;
    }
    double step = 1.0, step_used = 0.0;
    bool accepted = false;
    for (int bt = 0; bt <= max_backtracks; ++bt) {
      for (int i = 0; i < n; ++i) {
        double v = SCR(Y, i);
        if (__ldg(p.t.mass + i) == 0.0) v = __dadd_rn(v, __dmul_rn(step, SCR(delta, i)));
        SCR(cand, i) = v;
      }
      step_used = step;
      step = __dmul_rn(step, factor_bt);
      if (!alg_finite(p, ln, cand)) continue;
      alg_residual(p, ln, cand, rr, Gc);
      ++pc.trials;
      ++pc.rhs;
      if (!alg_finite(p, ln, Gc)) continue;
      if (alg_absmax(p, ln, Gc, red) == 0.0) {
        accepted = true;
        break;
      }
      solve_into(p, ln, lu, w, Gc, trial);
      ++pc.solves;
      if (!alg_finite(p, ln, trial)) continue;
      const double qt = weighted(p, ln, cand, trial, red);
      if (qt <= tol || qt < __dmul_rn(__dsub_rn(1.0, __dmul_rn(sigma, step_used)), q)) {
        accepted = true;
        break;
      }
    }
    if (!accepted) break;
    trace_record(p, g, nrec, 0.0, step_used, q, 2.0);
    for (int i = 0; i < n; ++i) SCR(Y, i) = SCR(cand, i);
  }
  if (have_orig)
    for (int i = 0; i < n; ++i) SCR(Y, i) = SCR(orig, i);
  return false;
}

// One group over one interval: fastode/solvers.py:305-415 statement by statement.
// The baseline restarting loop, fastode/solvers.py:205-267 statement by
// statement: a restart at 1e-6 of the interval, the elementary controller,
// no carried memory, "too many steps" past max_steps attempts.
__device__ __noinline__ void solve_group_restarting(const SolveParams& p, int g, double* scr, double* w,
                                                    double* red) {
  const int L = blockDim.x, lane = threadIdx.x;
  const int n = p.t.n;
  const int64_t c0 = p.group_offsets[g], C = p.group_offsets[g + 1] - c0;
  Lane ln;
  ln.lane = lane;
  ln.L = L;
  ln.active = lane < C;
  ln.cell = c0 + (ln.active ? lane : (C - 1));
  const DevOptions& o = p.o;
  const double dt = p.dt;
  long long c_steps = 0, c_acc = 0, c_rej = 0, c_rhs = 0, c_jac = 0, c_lu = 0, c_solves = 0;
  int nrec = 0;
  double* Y = scr + p.sl.y * L;
  double* Ynew = scr + p.sl.ynew * L;
  double* F0 = scr + p.sl.f0 * L;
  double* negj = scr + p.sl.negj * L;
  double* dd = scr + p.sl.d * L;
  double* rr = scr + p.sl.r * L;
  double* lu = scr + p.sl.lu * L;
  for (int i = 0; i < n; ++i) SCR(Y, i) = p.Y[ln.cell * p.ycs + (int64_t)__ldg(p.t.perm + i) * p.yss];
  const double rounding = 2.220446049250313e-16;
  const double h_min = __dmul_rn(1.0e-15, dt);
  const double h_max = dt;
  double H = pymin(pymax(h_min, __dmul_rn(1.0e-6, dt)), h_max);
  const double elem_exp = 1.0 / o.k_exp;
  const double nsize = (double)(C * n);
  int status = -1;
  ProjectionCounts pc;
  if (p.t.has_constraints && !project(p, ln, Y, scr, w, red, pc, g, nrec)) status = FO_STATUS_PROJECTION_FAILED;
  c_rhs += pc.rhs;
  c_jac += pc.jac;
  c_lu += pc.lu;
  c_solves += pc.solves;
  double t = 0.0;
  bool reject_last = false, reject_more = false;
  int nsteps = 0;
  while (status < 0 && __dadd_rn(__dsub_rn(t, dt), rounding) <= 0.0) {
    if (nsteps > o.max_steps) {
      status = FO_STATUS_TOO_MANY_STEPS;
      break;
    }
    if (__dadd_rn(t, __dmul_rn(0.1, H)) == t || H <= pymin(rounding, h_min)) {
      status = FO_STATUS_STEP_TOO_SMALL;
      break;
    }
    H = pymin(H, fabs(__dsub_rn(dt, t)));
    eval_rhs(p, ln, Y, rr, F0);
    ++c_rhs;
    eval_negjac(p, ln, Y, dd, negj);
    ++c_jac;
    bool accepted = false;
    while (!accepted) {
      factor_any(p, ln, 1.0 / __dmul_rn(H, o.tab.gamma), negj, lu, w, false);
      ++c_lu;
      const double total = block_sum(attempt(p, ln, H, Y, Ynew, scr, w, c_rhs, c_solves), red);
      double err = sqrt(__ddiv_rn(total, nsize));
      if (!isnan(err)) err = pymax(err, 1.0e-10);
      ++nsteps;
      ++c_steps;
      if (isnan(err) || isinf(err)) {
        trace_record(p, g, nrec, t, H, err, -1.0);
        status = FO_STATUS_NAN_OR_INF;
        break;
      }
      const double fac = pymin(6.0, pymax(0.2, __ddiv_rn(0.9, pow(err, elem_exp))));
      double Hnew = __dmul_rn(H, fac);
      if (err < 1.0 || H < h_min) {
        trace_record(p, g, nrec, t, H, err, 1.0);
        ++c_acc;
        t = __dadd_rn(t, H);
        double* tmp = Y;
        Y = Ynew;
        Ynew = tmp;
        Hnew = pymax(h_min, pymin(Hnew, h_max));
        if (reject_last) Hnew = pymin(Hnew, H);
        reject_last = reject_more = false;
        H = Hnew;
        accepted = true;
      } else {
        trace_record(p, g, nrec, t, H, err, 0.0);
        if (reject_more) Hnew = __dmul_rn(H, 0.1);
        reject_more = reject_last;
        reject_last = true;
        H = Hnew;
        ++c_rej;
      }
    }
  }
  if (status < 0) status = FO_STATUS_CONVERGED;
  const bool clamp = status != FO_STATUS_PROJECTION_FAILED;
  if (ln.active)
    for (int i = 0; i < n; ++i) {
      double y = SCR(Y, i);
      if (clamp && (!p.t.has_constraints || __ldg(p.t.mass + i) == 1.0)) y = clamp0(y);
      p.Y[ln.cell * p.ycs + (int64_t)__ldg(p.t.perm + i) * p.yss] = y;
    }
  if (threadIdx.x == 0) {
    long long* cn = p.counts + (int64_t)g * FO_NUM_COUNTS;
    cn[0] += c_steps;
    cn[1] += c_acc;
    cn[2] += c_rej;
    cn[3] += c_rhs;
    cn[4] += c_jac;
    cn[5] += c_lu;
    cn[6] += c_solves;
    cn[10] += pc.passes;
    cn[11] += pc.trials;
    cn[12] += 1;
    p.status[g] = status;
    if (p.trace_len) p.trace_len[g] = nrec;
  }
}

// The baseline backward Euler, fastode/solvers.py:439-491 statement by
// statement: every Newton iteration evaluates F and J at the iterate, factors
// M/H - J and solves for the update; the iterate is clamped at zero after
// each update. From the second iteration on, the step has converged when
// every update of the group is finite and within max(small, atol, rtol |Y|).
// A failed step restarts from the last accepted state with H cut by the next
// reduction; past the last reduction the unconverged iterate is accepted and
// the call ends. Two converged steps in a row double H.
__device__ __noinline__ void solve_group_backward_euler(const SolveParams& p, int g, double* scr, double* w,
                                                        double* red) {
  const int L = blockDim.x, lane = threadIdx.x;
  const int n = p.t.n;
  const int64_t c0 = p.group_offsets[g], C = p.group_offsets[g + 1] - c0;
  Lane ln;
  ln.lane = lane;
  ln.L = L;
  ln.active = lane < C;
  ln.cell = c0 + (ln.active ? lane : (C - 1));
  const DevOptions& o = p.o;
  const double dt = p.dt;
  long long c_steps = 0, c_acc = 0, c_rej = 0, c_rhs = 0, c_jac = 0, c_lu = 0, c_solves = 0;
  long long c_newton = 0, c_fail = 0, c_unconv = 0;
  double* Yn = scr + p.sl.y * L;
  double* Yn1 = scr + p.sl.ynew * L;
  double* F = scr + p.sl.f0 * L;
  double* negj = scr + p.sl.negj * L;
  double* dd = scr + p.sl.d * L;
  double* rr = scr + p.sl.r * L;
  double* lu = scr + p.sl.lu * L;
  const bool in_place = solves_in_place(p);   // Newton update solved in place in F
  for (int i = 0; i < n; ++i) {
    const double v = p.Y[ln.cell * p.ycs + (int64_t)__ldg(p.t.perm + i) * p.yss];
    SCR(Yn, i) = v;
    SCR(Yn1, i) = v;
  }
  double H = dt, t = 0.0;
  int n_success = 0, n_fail = 0;
  int status = FO_STATUS_CONVERGED;
  while (t < dt) {
    if (c_steps >= o.max_steps) {   // a guard of this build: the reference's loop has no budget
      status = FO_STATUS_TOO_MANY_STEPS;
      break;
    }
    bool ok = false;
    int iterations = 0;
    for (;;) {
      ++c_newton;
      eval_rhs(p, ln, Yn1, rr, F);
      ++c_rhs;
      eval_negjac(p, ln, Yn1, dd, negj);
      ++c_jac;
      factor_any(p, ln, 1.0 / H, negj, lu, w, false);
      ++c_lu;
      for (int i = 0; i < n; ++i) {
        const double v = __dsub_rn(SCR(F, i), __ddiv_rn(__dsub_rn(SCR(Yn1, i), SCR(Yn, i)), H));
        if (in_place) SCR(F, i) = v;
        else WROW(i) = v;
      }
      if (in_place) solve_into(p, ln, lu, w, F, F);
      else solve_in_w(p, ln, lu, w);
      ++c_solves;
      ++iterations;
      bool conv = true;
      for (int i = 0; i < n; ++i) {
        const double d = in_place ? SCR(F, i) : WROW(i);
        const double y = clamp0(__dadd_rn(SCR(Yn1, i), d));
        SCR(Yn1, i) = y;
        if (iterations > 1) {
          const double bound = npmax(npmax(o.small, __ldg(p.atol + __ldg(p.t.perm + i))), __dmul_rn(p.rtol, fabs(y)));
          conv = conv && isfinite(d) && fabs(d) <= bound;
        }
      }
      if (iterations > 1) ok = block_all(!ln.active || conv);
      if (ok || iterations >= o.max_iterations) break;
    }
    ++c_steps;
    if (!ok) {
      ++c_rej;
      ++c_fail;
      n_success = 0;
      if (n_fail >= o.nreductions) {
        t = __dadd_rn(t, H);
        ++c_unconv;
        status = FO_STATUS_ACCEPTED_UNCONVERGED;
        bool finite = true;
        for (int i = 0; i < n; ++i) finite = finite && isfinite(SCR(Yn1, i));
        if (!block_all(!ln.active || finite)) status = FO_STATUS_NAN_OR_INF;
        break;
      }
      for (int i = 0; i < n; ++i) SCR(Yn1, i) = SCR(Yn, i);
      H = __dmul_rn(H, o.reductions[n_fail]);
      ++n_fail;
    } else {
      ++c_acc;
      t = __dadd_rn(t, H);
      for (int i = 0; i < n; ++i) SCR(Yn, i) = SCR(Yn1, i);
      ++n_success;
      if (n_success >= 2) {
        n_success = 0;
        H = __dmul_rn(H, 2.0);
      }
    }
    H = pymin(H, __dsub_rn(dt, t));
  }
  if (ln.active)
    for (int i = 0; i < n; ++i) {
      double y = SCR(Yn1, i);
      if (!p.t.has_constraints || __ldg(p.t.mass + i) == 1.0) y = clamp0(y);
      p.Y[ln.cell * p.ycs + (int64_t)__ldg(p.t.perm + i) * p.yss] = y;
    }
  if (threadIdx.x == 0) {
    long long* cn = p.counts + (int64_t)g * FO_NUM_COUNTS;
    cn[0] += c_steps;
    cn[1] += c_acc;
    cn[2] += c_rej;
    cn[3] += c_rhs;
    cn[4] += c_jac;
    cn[5] += c_lu;
    cn[6] += c_solves;
    cn[7] += c_newton;
    cn[8] += c_fail;
    cn[9] += c_unconv;
    cn[12] += 1;
    p.status[g] = status;
    if (p.trace_len) p.trace_len[g] = 0;
  }
}

// Lockstep rounds. With every block of the launch resident at once (a
// cooperative launch), the groups make their attempts in rounds: each block
// makes one attempt (or p.round_attempts attempts, so that a round of a small
// mechanism costs about as much as one of the largest in a several-mechanism
// launch), then waits at a grid-wide barrier for the others; a block with no
// group left keeps arriving with nothing to do until a round in which no
// block attempted. The straight-line factorization is megabytes of code, so
// warps that drift apart each stream their own instructions and thrash the
// SM's instruction cache; rounds keep the warps of an SM at the same place
// (the cold first interval of the 210/500, 65,536-cell job: 1.47 s without
// rounds, 0.96 s with). The barrier only orders time: no group reads
// another's data, so results are those of the unsynchronized launch bit for
// bit. Each wait is bounded (kRoundSpinLimit polls about 4 us apart, some
// 30 s); a wait that gives up raises the give-up word, after which every
// block runs on without rounds.
constexpr long long kRoundSpinLimit = 7500000;

// Arrive with this block's activity in the round (1: it attempted); returns
// the number of blocks that attempted in the round, or -1 once rounds are
// given up. Barrier words: [0] arrivals, [1] activity sum, [2] generation,
// [3] the last round's sum, [4] give-up. Every thread of the block calls it.
__device__ int round_barrier(unsigned int* w, int active) {
  __shared__ int result;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* vw = w;
    if (vw[4] != 0u) {
      result = -1;
    } else {
      const unsigned int gen = vw[2];
      __threadfence();
      atomicAdd(w + 1, (unsigned int)active);
      __threadfence();
      if (atomicAdd(w, 1u) + 1u == gridDim.x) {
        const unsigned int total = atomicExch(w + 1, 0u);
        atomicExch(w + 3, total);
        atomicExch(w, 0u);
        __threadfence();
        atomicAdd(w + 2, 1u);
        result = (int)total;
      } else {
        long long spins = 0;
        while (vw[2] == gen && vw[4] == 0u && spins < kRoundSpinLimit) {
          __nanosleep(4000);
          ++spins;
        }
        __threadfence();
        if (vw[2] != gen) {
          result = (int)vw[3];
        } else {
          atomicExch(w + 4, 1u);
          result = -1;
        }
      }
    }
  }
  __syncthreads();
  return result;
}

// The parameters of batch b of a several-mechanism launch, copied from the
// batch table in global memory into the block's shared copy when the block
// moves to another batch, so that the integrator's parameter reads do not
// compete with the factorization's operand stream for L1. Every thread of
// the block calls this.
__device__ __forceinline__ void load_batch_params(const SolveParams* __restrict__ batches, int b, int& current,
                                                  SolveParams& shared) {
  static_assert(sizeof(SolveParams) % sizeof(long long) == 0, "SolveParams copies as 8-byte words");
  if (b == current) return;
  __syncthreads();
  const long long* src = reinterpret_cast<const long long*>(batches + b);
  long long* dst = reinterpret_cast<long long*>(&shared);
  for (int i = threadIdx.x; i < (int)(sizeof(SolveParams) / sizeof(long long)); i += blockDim.x) dst[i] = src[i];
  __syncthreads();
  current = b;
}

// A block with no group left: arrive idle until a round without attempts.
__device__ __forceinline__ void rounds_drain(unsigned int* w) {
  if (w != nullptr)
    while (round_barrier(w, 0) > 0) {
    }
}

__device__ void solve_group_algorithm(const SolveParams& p, int g, double* scr, double* w, double* red);

__device__ void solve_group(const SolveParams& p, int g, double* scr, double* w, double* red) {
  if (p.o.loop == FO_LOOP_RESTARTING) solve_group_restarting(p, g, scr, w, red);
  else if (p.o.loop == FO_LOOP_BACKWARD_EULER) solve_group_backward_euler(p, g, scr, w, red);
  else solve_group_algorithm(p, g, scr, w, red);
}

__device__ void solve_group_algorithm(const SolveParams& p, int g, double* scr, double* w, double* red) {
  const int L = blockDim.x, lane = threadIdx.x;
  const int n = p.t.n;
  const int64_t c0 = p.group_offsets[g], c1 = p.group_offsets[g + 1];
  const int64_t C = c1 - c0;
  Lane ln;
  ln.lane = lane;
  ln.L = L;
  ln.active = lane < C;
  ln.cell = c0 + (ln.active ? lane : (C - 1));
  const DevOptions& o = p.o;
  const double dt = p.dt;

  long long c_steps = 0, c_acc = 0, c_rej = 0, c_rhs = 0, c_jac = 0, c_lu = 0, c_solves = 0;
  int nrec = 0;
  int since_round = 0;

  double* Y = scr + p.sl.y * L;
  double* Ynew = scr + p.sl.ynew * L;
  double* F0 = scr + p.sl.f0 * L;
  double* negj = scr + p.sl.negj * L;
  double* dd = scr + p.sl.d * L;
  double* rr = scr + p.sl.r * L;
  double* lu = scr + p.sl.lu * L;

  for (int i = 0; i < n; ++i) SCR(Y, i) = p.Y[ln.cell * p.ycs + (int64_t)__ldg(p.t.perm + i) * p.yss];

  double* mem = p.memory + (int64_t)g * 3;
  double h_next = mem[0], err_prev = mem[1], h_prev = mem[2];
  if (!(o.carry && o.carry_memory)) err_prev = h_prev = 0.0;
  const double h_min = __dmul_rn(1.0e-15, dt);
  const double h_max = dt;
  double H = (o.carry && h_next > 0.0) ? h_next : __dmul_rn(1.0e-6, dt);
  H = pymin(pymax(h_min, H), h_max);
  if (o.quantize) H = quantize_step(H, dt);
  double proposed = H;
  const double elem_exp = 1.0 / o.k_exp;
  const double up = 1.0 + 1.0e-8, down = 1.0 - 1.0e-8;
  const double rounding = 2.220446049250313e-16;

  double t = 0.0;
  bool reject_last = false, reject_more = false;
  int nsteps = 0;
  int status = -1;  // running
  const double nsize = (double)(C * n);
  ProjectionCounts pc;
  if (p.t.has_constraints && !project(p, ln, Y, scr, w, red, pc, g, nrec)) {
    status = FO_STATUS_PROJECTION_FAILED;   // Y restored, no step taken
    proposed = h_next;                      // the carried proposal is left as it was
  }
  c_rhs += pc.rhs;
  c_jac += pc.jac;
  c_lu += pc.lu;
  c_solves += pc.solves;
  while (status < 0 && __dadd_rn(__dsub_rn(t, dt), rounding) <= 0.0) {
    if (nsteps >= o.max_steps) {
      status = FO_STATUS_TOO_MANY_STEPS;
      break;
    }
    if (__dadd_rn(t, __dmul_rn(0.1, H)) == t || H < h_min) {
      status = FO_STATUS_STEP_TOO_SMALL;
      break;
    }
    bool last = __dsub_rn(dt, t) <= __dmul_rn(H, up);
    bool shortened = last && __dsub_rn(dt, t) < __dmul_rn(H, down);
    double H_ctrl = H;
    if (last) H = __dsub_rn(dt, t);
    eval_rhs(p, ln, Y, rr, F0);
    ++c_rhs;
    eval_negjac(p, ln, Y, dd, negj);
    ++c_jac;
    bool accepted = false;
    while (!accepted) {
      if (nsteps >= o.max_steps) {
        status = FO_STATUS_TOO_MANY_STEPS;
        break;
      }
      if (H < h_min || __dadd_rn(t, __dmul_rn(0.1, H)) == t) {
        status = FO_STATUS_STEP_TOO_SMALL;
        break;
      }
      factor_any(p, ln, 1.0 / __dmul_rn(H, o.tab.gamma), negj, lu, w, false);
      ++c_lu;
      const double part = attempt(p, ln, H, Y, Ynew, scr, w, c_rhs, c_solves);
      const double total = block_sum(part, red);
      double err = sqrt(__ddiv_rn(total, nsize));
      if (!isnan(err)) err = pymax(err, 1.0e-10);
      ++nsteps;
      ++c_steps;
      if (isnan(err) || isinf(err)) {
        trace_record(p, g, nrec, t, H, err, -1.0);
        status = FO_STATUS_NAN_OR_INF;
        break;
      }
      if (err < 1.0 && shortened) {
        trace_record(p, g, nrec, t, H, err, 1.0);
        ++c_acc;
        t = dt;
        double* tmp = Y; Y = Ynew; Ynew = tmp;
        proposed = H_ctrl;
        accepted = true;
      } else if (err < 1.0) {
        trace_record(p, g, nrec, t, H, err, 1.0);
        // fastode/solvers.py:297-303
        double fac = __ddiv_rn(o.safety, pow(err, elem_exp));
        if (o.controller == FO_CONTROLLER_H211B && err_prev > 0.0 && h_prev > 0.0) {
          fac = __dmul_rn(__dmul_rn(o.safety, pow(__dmul_rn(err, err_prev), -1.0 / __dmul_rn(o.b, o.k_exp))),
                          pow(__ddiv_rn(H, h_prev), -1.0 / o.b));
        }
        fac = pymin(o.fac_max, pymax(o.fac_min, fac));
        ++c_acc;
        t = last ? dt : __dadd_rn(t, H);
        double* tmp = Y; Y = Ynew; Ynew = tmp;
        err_prev = err;
        h_prev = H;
        double Hnew = __dmul_rn(H, fac);
        if (reject_last) Hnew = pymin(Hnew, H);
        Hnew = pymax(h_min, pymin(Hnew, h_max));
        if (o.quantize) Hnew = quantize_step(Hnew, dt);
        reject_last = reject_more = false;
        proposed = Hnew;
        H = Hnew;
        accepted = true;
      } else {
        trace_record(p, g, nrec, t, H, err, 0.0);
        double Hnew = __dmul_rn(H, pymax(o.fac_min, __ddiv_rn(o.safety, pow(err, elem_exp))));
        if (reject_more) Hnew = __dmul_rn(H, 0.1);
        reject_more = reject_last;
        reject_last = true;
        if (o.quantize) Hnew = quantize_step(Hnew, dt);
        H = Hnew;
        last = __dsub_rn(dt, t) <= __dmul_rn(H, up);
        shortened = last && __dsub_rn(dt, t) < __dmul_rn(H, down);
        H_ctrl = H;
        if (last) H = __dsub_rn(dt, t);
        ++c_rej;
      }
      if (p.rounds != nullptr && ++since_round >= p.round_attempts) {
        since_round = 0;
        round_barrier(p.rounds, 1);
      }
    }
  }
  if (status < 0) status = FO_STATUS_CONVERGED;

  // clamp (fastode/solvers.py:89-97) and write back; a failed projection
  // returns the restored state unclamped (fastode/solvers.py:323-325)
  const bool clamp = status != FO_STATUS_PROJECTION_FAILED;
  if (ln.active) {
    for (int i = 0; i < n; ++i) {
      double y = SCR(Y, i);
      if (clamp && (!p.t.has_constraints || __ldg(p.t.mass + i) == 1.0)) y = clamp0(y);
      p.Y[ln.cell * p.ycs + (int64_t)__ldg(p.t.perm + i) * p.yss] = y;
    }
  }
  if (threadIdx.x == 0) {
    mem[0] = proposed;
    mem[1] = err_prev;
    mem[2] = h_prev;
    long long* cn = p.counts + (int64_t)g * FO_NUM_COUNTS;
    cn[0] += c_steps;
    cn[1] += c_acc;
    cn[2] += c_rej;
    cn[3] += c_rhs;
    cn[4] += c_jac;
    cn[5] += c_lu;
    cn[6] += c_solves;
    cn[10] += pc.passes;
    cn[11] += pc.trials;
    cn[12] += 1;
    p.status[g] = status;
    if (p.trace_len) p.trace_len[g] = nrec;
  }
}

}  // namespace
}  // namespace fo

