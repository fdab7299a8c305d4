// Discrete adjoint of the Rosenbrock steps on the device (no counterpart in the
// reference, which has no sensitivities).
//
// With the accepted step sizes of a forward run held fixed, one interval maps
// its start state Y_i (and the log rate constants) to its end state through
// the accepted steps of fastode/solvers.py:54-86 and the clamp of
// fastode/solvers.py:89-97. For each group, one block replays that map from the
// interval's checkpoint, keeping the state at the start of every step, then
// walks the steps backwards: it recomputes the step (Jacobian, factorization,
// stages) and runs the reverse stage sweep
//
//   mu_r   = A^-T Kbar_r                      (transposed solves with the same LU)
//   Fbar  += mu_r, Kbar_s += (c_rs/h) M mu_r  (s < r)
//   Jbar  += mu_r K_r^T                       (A = M/(h gamma) - J)
//   at every stage that evaluates F at its point u_r:
//       ybar += J(u_r)^T Fbar,  Kbar_s += a_rs J(u_r)^T Fbar,
//       logk_bar += r(u_r) * (S^T Fbar)
//   and finally the mass-action second derivatives of J(y) contracted with Jbar.
//
// Every lane is one cell (thread-per-cell, as in the forward kernels), so the
// per-cell gradient with respect to log k is written without atomics.
//
// Constrained systems start every call with the projection onto the
// algebraic constraints (fastode/solvers.py:100-178). Its accepted Newton
// updates y += s A(y)^-1 G(y) are replayed with the forward run's line-search
// steps s held fixed and reversed after the steps: mu = A^-T (s ybar), then
// ybar += (dG/dy)^T mu + (d(J_alg delta)/dy)^T mu (dA = -dJ_alg).
//
// This header holds the device functions; adjoint.cu launches them with the
// table-driven factorization and solves, generated.cu with a mechanism's
// generated ones (FO_LINK_GENERATED).
#pragma once

#include "rosenbrock.cuh"

namespace fo {
namespace {


// w[col[q]] -= lu[q] * z for q in [q0, q1): the factor entries of one row,
// loaded eight at a time before their updates so that their latencies
// overlap (the columns of one row are distinct, so the updates commute with
// the loads).
__device__ __forceinline__ void scatter_row(const double* __restrict__ lu, const int32_t* __restrict__ col, int q0,
                                            int q1, double z, double* w, int L, int lane) {
  constexpr int kBatch = 8;
  int q = q0;
  for (; q + kBatch <= q1; q += kBatch) {
    double v[kBatch];
    int c[kBatch];
#pragma unroll
    for (int i = 0; i < kBatch; ++i) {
      v[i] = SCR(lu, q + i);
      c[i] = __ldg(col + q + i);
    }
#pragma unroll
    for (int i = 0; i < kBatch; ++i) WROW(c[i]) = fma(-v[i], z, WROW(c[i]));
  }
  for (; q < q1; ++q) {
    const int c = __ldg(col + q);
    WROW(c) = fma(-SCR(lu, q), z, WROW(c));
  }
}

// Solve A^T x = b in place on w with the factors in lu (the diagonal slot
// holds 1/pivot): U^T z = b by columns of U, then L^T x = z by rows of L.
__device__ __noinline__ void lu_solve_transposed(const SolveParams& p, const Lane& ln, const double* lu, double* w) {
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n;
  const int32_t* __restrict__ rowp = p.t.lu_row_ptr;
  const int32_t* __restrict__ diag = p.t.lu_diag;
  const int32_t* __restrict__ col = p.t.lu_col;
  for (int r = 0; r < n; ++r) {
    const int dg = __ldg(diag + r), q1 = __ldg(rowp + r + 1);
    const double z = WROW(r) * SCR(lu, dg);
    WROW(r) = z;
    scatter_row(lu, col, dg + 1, q1, z, w, L, lane);
  }
  for (int r = n - 1; r >= 0; --r) {
    const double x = WROW(r);
    scatter_row(lu, col, __ldg(rowp + r), __ldg(diag + r), x, w, L, lane);
  }
}

// g = J(x)^T v for the mass-action forcing at x, and logk_bar += r(x) * (S^T v).
__device__ __noinline__ void vjp_forcing(const AdjParams& a, const Lane& ln, const double* x, const double* v,
                                         double* g) {
  const SolveParams& p = a.p;
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n, R = p.t.R, P = p.t.P;
  const double* kc = p.k + ln.cell * p.kcs;
  double* th = a.thbar + ln.cell * a.tcs;
  for (int i = 0; i < n; ++i) SCR(g, i) = 0.0;
  for (int j = 0; j < R; ++j) {
    double wj = 0.0;
    const int t1 = __ldg(p.t.st_ptr + j + 1);
    for (int t = __ldg(p.t.st_ptr + j); t < t1; ++t) wj = fma(__ldg(p.t.st_val + t), SCR(v, __ldg(p.t.st_sp + t)), wj);
    const double kj = __ldg(kc + (int64_t)j * p.krs);
    double rate = kj;
    for (int q = 0; q < P; ++q) {
      const int s = __ldg(p.t.react + j * P + q);
      if (s != n) rate *= SCR(x, s);
    }
    if (ln.active) th[(int64_t)j * a.trs] += wj * rate;
    for (int q = 0; q < P; ++q) {
      const int s = __ldg(p.t.react + j * P + q);
      if (s == n) continue;
      double d = kj;
      for (int q2 = 0; q2 < P; ++q2) {
        if (q2 == q) continue;
        const int s2 = __ldg(p.t.react + j * P + q2);
        if (s2 != n) d *= SCR(x, s2);
      }
      SCR(g, s) = fma(wj, d, SCR(g, s));
    }
  }
}

// ybar += grad_y sum_e Jbar_e J_e(y) and logk_bar += its log k derivative:
// J_e = sum of S[i,j] d[j,p] over the map's terms, d[j,p] = k_j prod_{q != p} y.
__device__ __noinline__ void hvp_jacobian(const AdjParams& a, const Lane& ln, const double* y, const double* jbar,
                                          double* dbar, double* ybar) {
  const SolveParams& p = a.p;
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n, R = p.t.R, P = p.t.P;
  const double* kc = p.k + ln.cell * p.kcs;
  double* th = a.thbar + ln.cell * a.tcs;
  for (int t = 0; t < R * P; ++t) SCR(dbar, t) = 0.0;
  for (int e = 0; e < p.t.nnzj; ++e) {
    const double je = SCR(jbar, e);
    const int t1 = __ldg(p.t.jt_ptr + e + 1);
    for (int t = __ldg(p.t.jt_ptr + e); t < t1; ++t) {
      const int jp = __ldg(p.t.jt_idx + t);
      SCR(dbar, jp) = fma(-__ldg(p.t.jt_val + t), je, SCR(dbar, jp));   // the map holds -S[i,j]
    }
  }
  for (int j = 0; j < R; ++j) {
    const double kj = __ldg(kc + (int64_t)j * p.krs);
    double th_j = 0.0;
    for (int q = 0; q < P; ++q) {
      if (__ldg(p.t.react + j * P + q) == n) continue;
      const double db = SCR(dbar, j * P + q);
      double d = kj;
      for (int q2 = 0; q2 < P; ++q2) {
        if (q2 == q) continue;
        const int s2 = __ldg(p.t.react + j * P + q2);
        if (s2 != n) d *= SCR(y, s2);
      }
      th_j = fma(db, d, th_j);
      for (int q2 = 0; q2 < P; ++q2) {
        if (q2 == q) continue;
        const int s2 = __ldg(p.t.react + j * P + q2);
        if (s2 == n) continue;
        double dd = kj;
        for (int q3 = 0; q3 < P; ++q3) {
          if (q3 == q || q3 == q2) continue;
          const int s3 = __ldg(p.t.react + j * P + q3);
          if (s3 != n) dd *= SCR(y, s3);
        }
        SCR(ybar, s2) = fma(db, dd, SCR(ybar, s2));
      }
    }
    if (ln.active) th[(int64_t)j * a.trs] += th_j;
  }
}

// The reverse sweep of one step whose forward pass left K_r and the stage
// points U_r in scratch and the factors of A(y) in lu; ybar holds dL/dy_new on
// entry and dL/dy on return.
__device__ __noinline__ void reverse_step(const AdjParams& a, const Lane& ln, double h, const double* y, double* scr,
                                          double* w) {
  const SolveParams& p = a.p;
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n;
  const DevTableau& tb = p.o.tab;
  const bool dae = p.t.has_constraints != 0;
  const double* K = scr + p.sl.k * L;
  const double* U = scr + a.al.u * L;
  const double* lu = scr + p.sl.lu * L;
  double* Kbar = scr + a.al.kbar * L;
  double* Fbar = scr + a.al.fbar * L;
  double* ybar = scr + a.al.ybar * L;
  double* g = scr + a.al.g * L;
  double* jbar = scr + a.al.jbar * L;
  double* dbar = scr + a.al.dbar * L;
  const int S = tb.S;
  for (int r = 0; r < S; ++r)
    for (int i = 0; i < n; ++i) {
      SCR(Kbar + (int64_t)r * n * L, i) = tb.m[r] * SCR(ybar, i);
      SCR(Fbar + (int64_t)r * n * L, i) = 0.0;
    }
  for (int e = 0; e < p.t.nnzj; ++e) SCR(jbar, e) = 0.0;
  for (int r = S - 1; r >= 0; --r) {
    int f = r;
    while (f > 0 && !tb.new_forcing[f]) --f;
#ifdef FO_LINK_GENERATED
    // the generated transposed solve works on the slot's solve vector
    double* muv = scr + p.sl.xs * L;
    for (int i = 0; i < n; ++i) SCR(muv, i) = SCR(Kbar + (int64_t)r * n * L, i);
    fo_gen_solve_t(scr + lane, p.o.gen_index);                           // mu_r
#else
    double* muv = w;
    for (int i = 0; i < n; ++i) WROW(i) = SCR(Kbar + (int64_t)r * n * L, i);
    lu_solve_transposed(p, ln, lu, w);                                   // w = mu_r
#endif
    const double* Kr = K + (int64_t)r * n * L;
    double coefs[4];                                                     // c(r, s) / h once per stage
    for (int s = 0; s < r; ++s) coefs[s] = tb.c[r][s] / h;
    for (int i = 0; i < n; ++i) {
      const double mu = SCR(muv, i);
      const int e1 = __ldg(p.t.j_row_ptr + i + 1);
      for (int e = __ldg(p.t.j_row_ptr + i); e < e1; ++e)
        SCR(jbar, e) = fma(mu, SCR(Kr, __ldg(p.t.j_col + e)), SCR(jbar, e));
      double* Ff = Fbar + (int64_t)f * n * L;
      SCR(Ff, i) += mu;
      for (int s = 0; s < r; ++s) {
        const double coef = coefs[s];
        if (coef != 0.0) {
          const double mv = dae ? mu * __ldg(p.t.mass + i) : mu;
          double* Ks = Kbar + (int64_t)s * n * L;
          SCR(Ks, i) = fma(coef, mv, SCR(Ks, i));
        }
      }
    }
    if (r == f) {
      const double* x = r == 0 ? y : U + (int64_t)r * n * L;
      vjp_forcing(a, ln, x, Fbar + (int64_t)f * n * L, g);
      for (int i = 0; i < n; ++i) {
        const double gi = SCR(g, i);
        SCR(ybar, i) += gi;
        for (int s = 0; s < r; ++s)
          if (tb.a[r][s] != 0.0) {
            double* Ks = Kbar + (int64_t)s * n * L;
            SCR(Ks, i) = fma(tb.a[r][s], gi, SCR(Ks, i));
          }
      }
    }
  }
  hvp_jacobian(a, ln, y, jbar, dbar, ybar);
}

// x = A^-T b with the factors in lu (b and x per-lane vectors; may alias).
__device__ void solve_transposed_into(const SolveParams& p, const Lane& ln, const double* lu, double* scr, double* w,
                                      const double* b, double* x) {
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n;
#ifdef FO_LINK_GENERATED
  double* v = scr + p.sl.xs * L;
  for (int i = 0; i < n; ++i) SCR(v, i) = SCR(b, i);
  fo_gen_solve_t(scr + lane, p.o.gen_index);
  for (int i = 0; i < n; ++i) SCR(x, i) = SCR(v, i);
#else
  for (int i = 0; i < n; ++i) WROW(i) = SCR(b, i);
  lu_solve_transposed(p, ln, lu, w);
  for (int i = 0; i < n; ++i) SCR(x, i) = WROW(i);
#endif
}

// The projection's Newton correction at y (fastode/solvers.py:110-124), the
// forward kernel's arithmetic exactly: G = F(y) on the algebraic rows, the
// algebraic-rows-only matrix A = diag(M) - J factored into lu, delta = A^-1 G.
__device__ void projection_delta(const AdjParams& a, const Lane& ln, const double* y, double* scr, double* w,
                                 double* delta) {
  const SolveParams& p = a.p;
  const int L = ln.L;
  double* G = scr + p.sl.f0 * L;
  double* negj = scr + p.sl.negj * L;
  double* lu = scr + p.sl.lu * L;
  alg_residual(p, ln, y, scr + p.sl.r * L, G);
  eval_negjac(p, ln, y, scr + p.sl.d * L, negj);
  factor_any(p, ln, 1.0, negj, lu, w, true);
  solve_into(p, ln, lu, w, G, delta);
}

// The reverse sweep of one projection update y' = y + s delta(y) (algebraic
// rows): with mu = A^-T (s ybar), ybar += J(y)^T mu_alg (delta's G) plus the
// second derivatives of J_alg contracted with mu delta^T (delta's matrix),
// and logk_bar gains the same terms' rate-constant derivatives. ybar holds
// dL/dy' on entry and dL/dy on return.
__device__ void reverse_projection_update(const AdjParams& a, const Lane& ln, double s, const double* y, double* scr,
                                          double* w) {
  const SolveParams& p = a.p;
  const int L = ln.L, lane = ln.lane;
  const int n = p.t.n;
  double* delta = scr + a.al.pdelta * L;
  double* mu = scr + a.al.pmu * L;
  double* ybar = scr + a.al.ybar * L;
  double* g = scr + a.al.g * L;
  double* jbar = scr + a.al.jbar * L;
  double* dbar = scr + a.al.dbar * L;
  projection_delta(a, ln, y, scr, w, delta);                       // lu: the factors of A(y)
  for (int i = 0; i < n; ++i) SCR(mu, i) = s * SCR(ybar, i);
  solve_transposed_into(p, ln, scr + p.sl.lu * L, scr, w, mu, mu);
  for (int i = 0; i < n; ++i) {
    const bool alg = __ldg(p.t.mass + i) == 0.0;
    const double m = SCR(mu, i);
    const int e1 = __ldg(p.t.j_row_ptr + i + 1);
    for (int e = __ldg(p.t.j_row_ptr + i); e < e1; ++e)
      SCR(jbar, e) = alg ? m * SCR(delta, __ldg(p.t.j_col + e)) : 0.0;
    if (!alg) SCR(mu, i) = 0.0;                                     // G has no differential rows
  }
  vjp_forcing(a, ln, y, mu, g);
  for (int i = 0; i < n; ++i) SCR(ybar, i) += SCR(g, i);
  hvp_jacobian(a, ln, y, jbar, dbar, ybar);
}

// One fixed step of size h from y (F, J, factorization, stages), the forward
// kernel's arithmetic exactly; y_new in ynew, stage points in U.
__device__ __forceinline__ void fixed_step(const AdjParams& a, const Lane& ln, double h, const double* y,
                                           double* ynew, double* scr, double* w, double* U) {
  const SolveParams& p = a.p;
  const int L = ln.L;
  long long cr = 0, cs = 0;
  eval_rhs(p, ln, y, scr + p.sl.r * L, scr + p.sl.f0 * L);
  eval_negjac(p, ln, y, scr + p.sl.d * L, scr + p.sl.negj * L);
  factor_any(p, ln, 1.0 / __dmul_rn(h, p.o.tab.gamma), scr + p.sl.negj * L, scr + p.sl.lu * L, w, false);
  attempt(p, ln, h, y, ynew, scr, w, cr, cs, U);
}

__device__ void adjoint_group(const AdjParams& a, double* w) {
  const SolveParams& p = a.p;
  const int L = blockDim.x, lane = threadIdx.x;
  const int g = blockIdx.x;
  const int n = p.t.n;
  const int64_t c0 = p.group_offsets[g], C = p.group_offsets[g + 1] - c0;
  Lane ln;
  ln.lane = lane;
  ln.L = L;
  ln.active = lane < C;
  ln.cell = c0 + (ln.active ? lane : (C - 1));
  double* scr = p.scratch + (int64_t)g * p.slot_doubles;
  const int s0 = a.step_ptr[g], m = a.step_ptr[g + 1] - s0;
  if (m > a.max_steps) {
    if (threadIdx.x == 0) a.status[g] = FO_STATUS_TOO_MANY_STEPS;
    return;
  }
  double* Y = scr + p.sl.y * L;
  double* Ynew = scr + p.sl.ynew * L;
  double* ys = scr + a.al.ys * L;
  double* U = scr + a.al.u * L;
  double* ybar = scr + a.al.ybar * L;
  for (int i = 0; i < n; ++i) SCR(Y, i) = a.Ycp[ln.cell * a.ycs + (int64_t)__ldg(p.t.perm + i) * a.yss];
  // replay the projection's updates (constrained systems), keeping the state
  // before each
  const int q0 = a.proj_ptr ? a.proj_ptr[g] : 0, nq = a.proj_ptr ? a.proj_ptr[g + 1] - q0 : 0;
  if (nq > kMaxProjectionUpdates) {
    if (threadIdx.x == 0) a.status[g] = FO_STATUS_PROJECTION_FAILED;
    return;
  }
  double* yp = scr + a.al.yp * L;
  for (int u = 0; u < nq; ++u) {
    double* yu = yp + (int64_t)u * n * L;
    double* delta = scr + a.al.pdelta * L;
    for (int i = 0; i < n; ++i) SCR(yu, i) = SCR(Y, i);
    projection_delta(a, ln, Y, scr, w, delta);
    const double st = a.proj_steps[q0 + u];
    for (int i = 0; i < n; ++i)
      if (__ldg(p.t.mass + i) == 0.0) SCR(Y, i) = __dadd_rn(SCR(Y, i), __dmul_rn(st, SCR(delta, i)));
  }
  // replay the accepted steps, keeping the state at the start of each
  for (int s = 0; s < m; ++s) {
    for (int i = 0; i < n; ++i) SCR(ys + (int64_t)s * n * L, i) = SCR(Y, i);
    fixed_step(a, ln, a.steps[s0 + s], Y, Ynew, scr, w, U);
    double* t = Y;
    Y = Ynew;
    Ynew = t;
  }
  const bool constrained = p.t.has_constraints != 0;
  if (a.mode == 0) {
    if (ln.active)
      for (int i = 0; i < n; ++i) {
        double y = SCR(Y, i);
        if (!constrained || __ldg(p.t.mass + i) == 1.0) y = clamp0(y);
        a.Yout[ln.cell * a.ocs + (int64_t)__ldg(p.t.perm + i) * a.oss] = y;
      }
    if (threadIdx.x == 0) a.status[g] = FO_STATUS_CONVERGED;
    return;
  }
  // dL/dY at the end of the interval through the clamp
  for (int i = 0; i < n; ++i) {
    double lam = a.lam[ln.cell * a.lcs + (int64_t)__ldg(p.t.perm + i) * a.lss];
    if ((!constrained || __ldg(p.t.mass + i) == 1.0) && !(SCR(Y, i) > 0.0)) lam = 0.0;
    SCR(ybar, i) = lam;
  }
  for (int s = m - 1; s >= 0; --s) {
    const double h = a.steps[s0 + s];
    const double* y = ys + (int64_t)s * n * L;
    fixed_step(a, ln, h, y, Ynew, scr, w, U);
    reverse_step(a, ln, h, y, scr, w);
  }
  for (int u = nq - 1; u >= 0; --u)
    reverse_projection_update(a, ln, a.proj_steps[q0 + u], yp + (int64_t)u * n * L, scr, w);
  bool finite = true;
  for (int i = 0; i < n; ++i) {
    const double v = SCR(ybar, i);
    if (!isfinite(v)) finite = false;
    if (ln.active) a.lam[ln.cell * a.lcs + (int64_t)__ldg(p.t.perm + i) * a.lss] = v;
  }
  finite = __syncthreads_and(finite ? 1 : 0) != 0;
  if (threadIdx.x == 0) a.status[g] = finite ? FO_STATUS_CONVERGED : FO_STATUS_NAN_OR_INF;
}

}  // namespace
}  // namespace fo
