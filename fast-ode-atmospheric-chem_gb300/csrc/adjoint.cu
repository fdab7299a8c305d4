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
#include <cuda_runtime.h>

#include "rosenbrock.cuh"

namespace fo {

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
    for (int i = 0; i < n; ++i) WROW(i) = SCR(Kbar + (int64_t)r * n * L, i);
    lu_solve_transposed(p, ln, lu, w);                                   // w = mu_r
    const double* Kr = K + (int64_t)r * n * L;
    for (int i = 0; i < n; ++i) {
      const double mu = WROW(i);
      const int e1 = __ldg(p.t.j_row_ptr + i + 1);
      for (int e = __ldg(p.t.j_row_ptr + i); e < e1; ++e)
        SCR(jbar, e) = fma(mu, SCR(Kr, __ldg(p.t.j_col + e)), SCR(jbar, e));
      double* Ff = Fbar + (int64_t)f * n * L;
      SCR(Ff, i) += mu;
      for (int s = 0; s < r; ++s) {
        const double coef = tb.c[r][s] / h;
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

__global__ void __maxnreg__(255) adjoint_kernel(AdjParams a) {
  extern __shared__ double smem[];
  double* red = smem;
  double* w = smem + 32;
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
  bool finite = true;
  for (int i = 0; i < n; ++i) {
    const double v = SCR(ybar, i);
    if (!isfinite(v)) finite = false;
    if (ln.active) a.lam[ln.cell * a.lcs + (int64_t)__ldg(p.t.perm + i) * a.lss] = v;
  }
  finite = __syncthreads_and(finite ? 1 : 0) != 0;
  if (threadIdx.x == 0) a.status[g] = finite ? FO_STATUS_CONVERGED : FO_STATUS_NAN_OR_INF;
}

cudaError_t launch_adjoint(const AdjParams& a, int grid, int lanes, size_t smem, cudaStream_t stream) {
  static int configured_smem = -1;
  if ((int)smem > 48 * 1024 && (int)smem != configured_smem) {
    cudaError_t e = cudaFuncSetAttribute(adjoint_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured_smem = (int)smem;
  }
  adjoint_kernel<<<grid, lanes, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace fo
