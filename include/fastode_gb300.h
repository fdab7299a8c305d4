/*
 * fastode_gb300 — C-ABI of the GB300 Rosenbrock integrator for mass-action
 * chemistry (FP64, sm_103a).
 *
 * This header is the drop-in boundary for the reference package fastode
 * (davidfillmore/Fast-ODE-Atmospheric-Chem). Each entry point names the
 * reference interface it replaces. All functions return an int status
 * (FO_OK = 0 or a negative FO_E* code) and never abort; numerical failures
 * of an integration are reported per group in the status array, with the
 * codes of FO_STATUS_*, exactly as the reference returns status strings.
 *
 * Data layout on the device: a state array Y holds n species x C cells and a
 * rate-constant array k holds R reactions x C cells. Both are addressed by
 * two strides (in doubles): element (cell c, species s) is at
 * Y[c * y_cell_stride + s * y_species_stride]. The batched layout is
 * species-major with cells fastest (cell stride 1, species stride C), which
 * makes every warp access a coalesced 256-byte line; the reference's (C, n)
 * row-major layout is cell stride n, species stride 1.
 *
 * Pointers marked "device" must be device memory (cudaMalloc or a torch CUDA
 * tensor); "host" pointers are host memory. The stream argument is a
 * cudaStream_t passed as void* (0 = legacy default stream).
 */
#ifndef FASTODE_GB300_H
#define FASTODE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FO_OK 0
#define FO_E_INVALID (-1)      /* bad argument */
#define FO_E_CUDA (-2)         /* a CUDA runtime call failed */
#define FO_E_UNSUPPORTED (-3)  /* size or option outside what the kernels handle */
#define FO_E_WORKSPACE (-4)    /* workspace too small */
#define FO_E_ALLOC (-5)        /* host allocation failed */

/* Per-group integration status; the strings are those of fastode/solvers.py:305-415. */
#define FO_STATUS_CONVERGED 0          /* "converged" */
#define FO_STATUS_TOO_MANY_STEPS 1     /* "too many steps" */
#define FO_STATUS_STEP_TOO_SMALL 2     /* "step too small" */
#define FO_STATUS_NAN_OR_INF 3         /* "nan or inf" */
#define FO_STATUS_PROJECTION_FAILED 4  /* "projection failed" */
#define FO_STATUS_ACCEPTED_UNCONVERGED 5  /* "accepted unconverged" (backward Euler, fastode/solvers.py:470-478) */

/* Number and order of the per-group counters (fastode/counts.py:10-23):
 * steps, accepted, rejected, rhs, jac, lu, solves, newton, failures,
 * unconverged, proj_passes, proj_trials, calls. */
#define FO_NUM_COUNTS 13

/* Tableaus (fastode/tableaus.py:70-90). */
#define FO_TABLEAU_ROS3 0
#define FO_TABLEAU_RODAS3 1

/* Step-size controllers of fastode/solvers.py:297-303. */
#define FO_CONTROLLER_H211B 0
#define FO_CONTROLLER_ELEMENTARY 1

/* Fill-reducing orderings for the pivot-free sparse LU. AUTO takes the greedy
 * order (natural, minimum degree, minimum fill) with the fewest LU FMAs and
 * refines it by a deterministic local search on the FMA count (about a second
 * of host time for 210 species); REFINED is AUTO reported as such even when
 * the search finds nothing better. */
#define FO_ORDER_AUTO 0
#define FO_ORDER_NATURAL 1
#define FO_ORDER_MIN_DEGREE 2
#define FO_ORDER_MIN_FILL 3
#define FO_ORDER_REFINED 4

/*
 * A compiled mechanism, as fastode.chem.Mechanism builds it
 * (fastode/chem.py:19-79): reactant table, stoichiometry, Jacobian pattern
 * and the sparse map from rate partials to Jacobian values. All host pointers.
 */
typedef struct fo_mechanism_desc {
  int32_t n;                  /* species */
  int32_t R;                  /* reactions */
  int32_t P;                  /* reactant slots per reaction */
  const int64_t* react;       /* R*P row-major species indices; n pads a slot (a factor of one) */
  const int32_t* s_indptr;    /* n+1: stoichiometry rows S[i, :] in CSR */
  const int32_t* s_idx;       /* reaction index of each nonzero */
  const double* s_val;        /* S[i, j] */
  int32_t nnz;                /* Jacobian pattern entries (diagonal included) */
  const int64_t* pat_rows;    /* nnz */
  const int64_t* pat_cols;    /* nnz */
  const int32_t* j_indptr;    /* nnz+1: Jacobian-value map in CSR over entries (the GT map) */
  const int32_t* j_idx;       /* j*P + p of each term */
  const double* j_val;        /* coefficient S[i, j] of each term */
  const double* mass;         /* n: 1 differential, 0 algebraic (may be NULL: all ones) */
} fo_mechanism_desc;

/* What the symbolic analysis found (host-side, no GPU needed). */
typedef struct fo_plan_info {
  int32_t n, R, P, nnz_jac;
  int32_t ordering;           /* the FO_ORDER_* actually used */
  int32_t nnz_lu;             /* entries of L+U including the diagonal (pattern plus fill) */
  int32_t nnz_l, nnz_u;       /* strictly lower / strictly upper entries */
  int64_t lu_fma;             /* multiply-adds of one factorization */
  int64_t solve_fma;          /* multiply-adds of one forward+backward solve */
  int32_t jac_terms;          /* terms of the Jacobian-value map */
  int32_t stoich_nnz;         /* nonzeros of S */
  int64_t scratch_doubles_per_cell;  /* per-cell device scratch of the integrator */
  int32_t smem_doubles_per_cell;     /* per-cell shared memory of the integrator */
  int32_t compact_smem_doubles_per_cell;  /* the same for FO_VARIANT_COMPACT */
} fo_plan_info;

typedef struct fo_plan fo_plan;  /* opaque */

/* Integrator options: the constructor arguments of fastode.Algorithm
 * (fastode/solvers.py:275-292). */
typedef struct fo_options {
  int32_t tableau;            /* FO_TABLEAU_* */
  int32_t controller;         /* FO_CONTROLLER_* ("h211b" or anything else = elementary) */
  double b;                   /* filter parameter (4) */
  double safety;              /* 0.9 */
  double fac_min;             /* 0.2 */
  double fac_max;             /* 6 */
  int32_t carry;              /* start from the carried proposal */
  int32_t quantize;           /* round proposals to divisors of the interval */
  int32_t carry_memory;       /* keep the filter memory across intervals */
  int32_t max_steps;          /* attempt budget per call (1000) */
  int32_t variant;            /* FO_VARIANT_*: which LU/solve kernel (same results up to roundoff) */
  int32_t loop;               /* FO_LOOP_*: the step loop */
  int32_t step_change_rows;   /* restarting loop with constraints: the step change replaces the
                                 algebraic rows of the error estimate (fastode/solvers.py:194-200) */
  /* Backward Euler (FO_LOOP_BACKWARD_EULER): the constructor arguments of
   * fastode.solvers.BackwardEuler (fastode/solvers.py:418-430). */
  int32_t max_iterations;     /* Newton iterations per step (11) */
  int32_t nreductions;        /* entries of reductions used, 0..8 (5) */
  double reductions[8];       /* step factor after the i-th failed step (0.5, 0.5, 0.5, 0.5, 0.1); each > 0 */
  double small;               /* floor of the convergence bound (1e-40) */
  /* Nonzero: with FO_VARIANT_GENERATED and FO_LOOP_ALGORITHM, when every
   * block of the launch is resident at once, fo_solve and fo_multi_launch
   * make the groups' attempts in rounds (one attempt per block, then a
   * grid-wide barrier) in a cooperative launch, which keeps the warps of an
   * SM in the same part of the generated code. Results are the same bit for
   * bit; otherwise the groups run unsynchronized. */
  int32_t lockstep;
} fo_options;

/* Step loops. ALGORITHM is fastode.solvers.Algorithm (fastode/solvers.py:270-415);
 * RESTARTING is the baseline fastode.solvers.RestartingLoop (fastode/solvers.py:189-267):
 * a restart at 1e-6 of the interval every call, the elementary controller, no
 * carried memory (b, fac_min, fac_max, carry, quantize, carry_memory and the
 * memory array are ignored; the memory array is neither read nor written). */
#define FO_LOOP_ALGORITHM 0
#define FO_LOOP_RESTARTING 1
/* BACKWARD_EULER is the baseline fastode.solvers.BackwardEuler
 * (fastode/solvers.py:418-491): backward Euler with a full Newton iteration
 * (rhs, Jacobian, factorization of M/H - J and one solve per iteration), the
 * step cut by reductions[i] after the i-th failed Newton iteration and doubled
 * after two converged steps in a row; past nreductions failures the last
 * iterate is accepted and the group reports FO_STATUS_ACCEPTED_UNCONVERGED.
 * It uses max_iterations, nreductions, reductions, small and max_steps; the
 * tableau must still name a valid tableau (it is not used), and the memory
 * array is neither read nor written. max_steps has no counterpart in the
 * reference, whose loop has no budget: it only guards against step
 * sequences that would not end (a group past it reports
 * FO_STATUS_TOO_MANY_STEPS). */
#define FO_LOOP_BACKWARD_EULER 2

/* Kernel variants of the factorization and solves. GENERATED (below) is the
 * fastest, for groups of up to 32 cells, and the default of the Python
 * layer; the table-driven ones serve larger groups: PIPELINED streams the
 * elimination schedule in hazard-free chunks through a shared-memory operand
 * ring, with the whole compressed row on chip; PLAIN is the direct
 * row-by-row loop, kept as the baseline it is measured against; COMPACT
 * (below) is the fastest table-driven one where its tables fit. */
#define FO_VARIANT_PIPELINED 0
#define FO_VARIANT_PLAIN 1
/* COMPACT eliminates every row in two passes over halves of its slots (the
 * second pass reloads the first pass's multipliers) and solves with half the
 * vector staged at a time, the other half in global memory, so a group needs
 * about half the shared memory and twice as many groups stay resident per SM.
 * The factors are those of PIPELINED bit for bit; the solves differ in
 * summation order (roundoff). fo_adjoint_interval runs PIPELINED for COMPACT
 * (its transposed solves need the whole vector on chip) and the generated
 * adjoint for GENERATED. */
#define FO_VARIANT_COMPACT 2
/* GENERATED runs the mechanism's own factorization and solves, generated as
 * straight-line code from its fill pattern and compiled when the plan is
 * prepared with fo_plan_generate (register tiles of the factorization, every
 * operand at an immediate offset, no schedule tables). Groups of at most 32
 * cells. Factors and solutions are those of PLAIN bit for bit. */
#define FO_VARIANT_GENERATED 3

/* What fo_plan_generate did. */
typedef struct {
  int32_t from_cache;    /* 1: the linked module was read from the cache */
  int32_t registers;     /* registers per thread of the generated kernel */
  int32_t tile;          /* rows and columns of the factorization's register tiles */
  int32_t local_bytes;   /* local memory per thread (spills) of the generated kernel */
  double seconds;        /* host time: generation, linking (or cache read) and loading */
  int64_t ptx_bytes;     /* size of the generated PTX */
  int64_t cubin_bytes;   /* size of the linked module */
} fo_gen_info;

/* Host-only symbolic analysis: ordering, fill and flop counts, and (when
 * perm is not NULL) the elimination order perm[p] = species eliminated p-th.
 * Replaces the ordering step of SuperLU's splu(permc_spec="MMD_AT_PLUS_A")
 * that fastode/linalg.py:70-78 runs on every factorization. Needs no GPU. */
int fo_analyze(const fo_mechanism_desc* mech, int32_t ordering, fo_plan_info* info, int32_t* perm);

/* Build a plan: symbolic analysis on the host, then the index tables are
 * copied to the current CUDA device. Replaces fastode.chem.Mechanism's
 * compiled tables (fastode/chem.py:19-79) plus linalg.SparsePattern
 * (fastode/linalg.py:32-67) as the device sees them. */
int fo_plan_create(const fo_mechanism_desc* mech, int32_t ordering, fo_plan** plan);
int fo_plan_info_get(const fo_plan* plan, fo_plan_info* info);
int fo_plan_destroy(fo_plan* plan);

/* The permutation chosen by the ordering: perm[p] = species eliminated p-th (host, n). */
int fo_plan_permutation(const fo_plan* plan, int32_t* perm);

/* Prepare a plan for FO_VARIANT_GENERATED: generate the mechanism's
 * factorization of alpha*M - J and its triangular solves as straight-line PTX
 * from the plan's fill pattern (the per-mechanism form of
 * fastode/linalg.py:70-81 and of the Jacobian assembly of
 * fastode/linalg.py:60-67), link it with the library's integrator kernel
 * (nvJitLink, opened at run time) and load the module on the current device.
 * The linked module is cached in cache_dir under a hash of its inputs (NULL:
 * $FASTODE_GB300_CACHE, else $XDG_CACHE_HOME/fastode_gb300, else
 * ~/.cache/fastode_gb300; "": no cache). Linking compiles the generated code:
 * about a minute for 200,000 multiply-adds; a cached module loads in
 * milliseconds. info may be NULL. Idempotent. Returns FO_E_UNSUPPORTED when
 * nvJitLink is missing or linking fails (fo_last_error has the log). */
int fo_plan_generate(fo_plan* plan, const char* cache_dir, fo_gen_info* info);

/* The generated code's shape for this plan, before fo_plan_generate (and
 * before the plan joins a generated several-mechanism launch): the rows and
 * columns of the factorization's register tiles (1..16, default 6) and the
 * rows of a block of the solves (1..64, default 8). A tuning choice that
 * changes no result: every tile gives the same factors bit for bit. Refused
 * once the plan's module exists with other options. */
int fo_plan_set_generation(fo_plan* plan, int32_t tile, int32_t solve_block);

/* Host-only check of the generated variant (no device needed): generate the
 * mechanism's code for the given ordering and, when link is nonzero, link it
 * with the integrator (nvJitLink); info gets the sizes and the time taken
 * (default tile and solve block). No counterpart in the reference. */
int fo_generate_check(const fo_mechanism_desc* mech, int32_t ordering, int32_t link, fo_gen_info* info);

/* Bytes of device workspace fo_solve needs for `slots` groups in flight
 * of at most `max_group_cells` cells each (see fo_solve). */
int fo_workspace_bytes(const fo_plan* plan, int32_t slots, int32_t max_group_cells, size_t* bytes);

/*
 * Integrate every group over one interval of length dt: the device form of
 * fastode.solvers.Algorithm.solve(system, Y, dt, atol, rtol, counts, memory)
 * (fastode/solvers.py:305-415), for many groups at once.
 *
 * Group g holds cells [group_offsets[g], group_offsets[g+1]) and shares one
 * step sequence, one error norm and one controller memory, as a group of C
 * cells shares them in the reference. group_offsets (device, ngroups+1) must
 * be increasing; no group may hold more than max_group_cells cells, and
 * max_group_cells may be 1..256 (n * roundup32(max_group_cells) doubles must
 * fit in shared memory).
 *
 * Y          device, in/out, updated in place to the clamped result.
 * k          device, rate constants (C x R via the two k strides).
 * atol       device, n doubles (species order of the mechanism).
 * memory     device, ngroups x 3 doubles (h_next, err_prev, h_prev) in/out
 *            (fastode/solvers.py:181-186 Memory).
 * counts     device, ngroups x FO_NUM_COUNTS int64, ACCUMULATED (+=).
 * status     device, ngroups int32, written (FO_STATUS_*).
 * workspace  device, at least fo_workspace_bytes(plan, slots, max_cells).
 * slots      groups integrated concurrently: 0 launches one block per group;
 *            a positive value launches that many persistent blocks that pull
 *            groups from a device queue.
 * trace      device or NULL: per group, trace_cap records of 4 doubles
 *            (t, H, err, outcome: 1 accepted, 0 rejected, -1 failed);
 *            trace_len (device, ngroups int32) receives the record count.
 */
int fo_solve(const fo_plan* plan, const fo_options* opt,
             int32_t ngroups, const int32_t* group_offsets, int32_t max_group_cells,
             double* Y, int64_t y_cell_stride, int64_t y_species_stride,
             const double* k, int64_t k_cell_stride, int64_t k_reaction_stride,
             const double* atol, double rtol, double dt,
             double* memory, int64_t* counts, int32_t* status,
             void* workspace, size_t workspace_bytes, int32_t slots,
             double* trace, int32_t trace_cap, int32_t* trace_len,
             void* stream);

/*
 * Several mechanisms in one persistent launch. Each batch is what one
 * fo_solve call takes (a plan, its options and groups, its state, rate
 * constants, tolerances, memory, counters and statuses, all device
 * pointers); the launch's blocks pull groups of every batch from one device
 * queue, largest mechanisms first. The device form of running the reference's
 * scenario loop (fastode/ts1.py:196-222) over several mechanisms at once.
 *
 * fo_multi_prepare validates the batches, checks the workspace (see
 * fo_multi_workspace_bytes) and writes the batch table into it (synchronous);
 * fo_multi_launch then only resets the queue and launches, so it can be
 * captured in a CUDA graph and replayed once per interval. The pointers given
 * to prepare must stay valid for every launch. With FO_VARIANT_GENERATED in
 * every batch (groups of at most 32 cells), prepare generates and links one
 * module holding every distinct mechanism's factorization and solves (the
 * default cache of fo_plan_generate applies) and the launch runs it; a mix of
 * generated and table-driven batches is refused (FO_E_UNSUPPORTED).
 */
typedef struct fo_batch_desc {
  const fo_plan* plan;
  fo_options opt;
  int32_t ngroups;
  const int32_t* group_offsets;   /* device, ngroups+1 */
  int32_t max_group_cells;        /* 1..256 */
  double* Y;
  int64_t y_cell_stride, y_species_stride;
  const double* k;
  int64_t k_cell_stride, k_reaction_stride;
  const double* atol;
  double rtol, dt;
  double* memory;
  int64_t* counts;
  int32_t* status;
} fo_batch_desc;

typedef struct fo_multi fo_multi;  /* opaque */

int fo_multi_workspace_bytes(int32_t nbatches, const fo_batch_desc* batches, int32_t slots, size_t* bytes);
int fo_multi_prepare(int32_t nbatches, const fo_batch_desc* batches, void* workspace, size_t workspace_bytes,
                     int32_t slots, fo_multi** multi);
int fo_multi_launch(const fo_multi* multi, void* stream);
int fo_multi_destroy(fo_multi* multi);

/* Photolysis update reading the time from device memory (t_dev, one double),
 * and a clock advance t_dev += dt: together they make an interval's launches
 * independent of the interval index, so one captured CUDA graph serves every
 * interval (fastode/ts1.py:204 evaluates the factor at the interval start). */
int fo_update_photolysis_clock(int32_t C, int32_t nphoto, const int32_t* rxn, const double* J,
                               const double* phase, double omega, const double* t_dev, double* k,
                               int64_t k_cell_stride, int64_t k_reaction_stride, void* stream);
int fo_advance_clock(double* t_dev, double dt, void* stream);

/*
 * Discrete adjoint of one interval (no counterpart in the reference, which has
 * no sensitivities). With the accepted step sizes of a forward run held fixed
 * (steps[step_ptr[g] .. step_ptr[g+1]) for group g, in order), the interval
 * maps its start state Y (the checkpoint, device) and the log rate constants
 * to its clamped end state through the steps of fastode/solvers.py:54-97.
 *
 * mode 0 (replay): writes that end state into Yout — the fixed-step map that
 *        finite differences are taken of.
 * mode 1 (adjoint): lam holds dL/dY at the interval end on entry and dL/dY at
 *        the interval start on return; thbar (C x R via its strides) gains
 *        dL/dlog k of every cell and reaction.
 * Groups with more than max_steps steps get FO_STATUS_TOO_MANY_STEPS; a
 * non-finite adjoint FO_STATUS_NAN_OR_INF. Workspace: fo_adjoint_workspace_bytes.
 * One block per group. Constrained systems (mass 0 rows): the consistent-
 * initialization projection that starts every call (fastode/solvers.py:100-178)
 * is part of the map and is differentiated too. proj_steps[proj_ptr[g] ..
 * proj_ptr[g+1]) are the line-search steps of the Newton updates the forward
 * call applied to group g, in order (its trace's records of outcome 2); the
 * updates are replayed with those steps held fixed and their reverse sweep is
 * a transposed solve with the projection's matrix, the forcing's
 * vector-Jacobian product and the Jacobian's second derivatives. NULL, NULL:
 * no updates (required for unconstrained mechanisms).
 */
int fo_adjoint_workspace_bytes(const fo_plan* plan, int32_t ngroups, int32_t max_group_cells, int32_t max_steps,
                               size_t* bytes);
int fo_adjoint_interval(const fo_plan* plan, const fo_options* opt, int32_t ngroups, const int32_t* group_offsets,
                        int32_t max_group_cells,
                        const double* Y, int64_t y_cell_stride, int64_t y_species_stride,
                        const double* k, int64_t k_cell_stride, int64_t k_reaction_stride,
                        const double* atol, double dt,
                        const int32_t* step_ptr, const double* steps, int32_t max_steps,
                        const int32_t* proj_ptr, const double* proj_steps, int32_t mode,
                        double* lam, int64_t lam_cell_stride, int64_t lam_species_stride,
                        double* thbar, int64_t thbar_cell_stride, int64_t thbar_reaction_stride,
                        double* Yout, int64_t yout_cell_stride, int64_t yout_species_stride,
                        int32_t* status, void* workspace, size_t workspace_bytes, void* stream);

/* Forcing F(Y) (C x n, written with the Y strides into F) for C cells:
 * fastode.chem.Mechanism.rhs (fastode/chem.py:89-90). Device pointers. */
int fo_eval_rhs(const fo_plan* plan, int32_t C,
                const double* Y, int64_t y_cell_stride, int64_t y_species_stride,
                const double* k, int64_t k_cell_stride, int64_t k_reaction_stride,
                double* F, void* stream);

/* Jacobian values on the mechanism's pattern, C x nnz row-major:
 * fastode.chem.Mechanism.jac_values (fastode/chem.py:92-102). Device pointers. */
int fo_eval_jac(const fo_plan* plan, int32_t C,
                const double* Y, int64_t y_cell_stride, int64_t y_species_stride,
                const double* k, int64_t k_cell_stride, int64_t k_reaction_stride,
                double* J, void* stream);

/* Thermal rate constants on the device: k[c, j] = A[j] exp(-E[j] / T[c]) *
 * M[c]^power[j] (power may be NULL: no third bodies). The Arrhenius rows of
 * fastode.ts1.TS1.rate_constants (fastode/ts1.py:76-79) with [M] folded in as
 * fastode/ts1.py:100-102 folds it. Device pointers; asynchronous on stream. */
int fo_rate_constants(int32_t C, int32_t R, const double* A, const double* E, const double* power,
                      const double* T, const double* M, double* k,
                      int64_t k_cell_stride, int64_t k_reaction_stride, void* stream);

/* Photolysis columns at an interval start: k[c, rxn[p]] = J[p] *
 * max(0, cos(phase[c] + omega * t)), the device form of the per-interval
 * photolysis patch of fastode/ts1.py:204-214. Device pointers; asynchronous. */
int fo_update_photolysis(int32_t C, int32_t nphoto, const int32_t* rxn, const double* J,
                         const double* phase, double omega, double t, double* k,
                         int64_t k_cell_stride, int64_t k_reaction_stride, void* stream);

/* Rate laws of a mechanism's reactions, evaluated per cell on the device
 * (fastode.ts1.TS1.rate_constants, fastode/ts1.py:66-103), in the
 * reference's operation order; T in K, P in Pa, M = P / (R T) in mol m^-3.
 *   FO_RATE_ARRHENIUS  k = A exp(C / T) (T / D)^B (1 + E P);
 *                      c = {A, B, C, D, E}
 *   FO_RATE_TROE       k0 = A0 exp(C0 / T) (T / 300)^B0, kinf likewise,
 *                      r = k0 M / kinf, k = k0 M / (1 + r) Fc^(N / (N + log10(r)^2));
 *                      c = {A0, B0, C0, Ainf, Binf, Cinf, Fc, N}
 *   FO_RATE_USER       k = param[column] * c[0] (the scaling factor)
 *   FO_RATE_SURFACE    v = sqrt(c[0] T) with c[0] = 8 R / (pi mw),
 *                      k = 4 n pi r^2 / (r / c[1] + 4 / (v c[2])), r the
 *                      effective radius (param[column]), n the particle number
 *                      concentration (param[column + 1]), c[1] the gas-phase
 *                      diffusion coefficient, c[2] the reaction probability
 * A scalar exponent of -1, 0, 0.5, 1 or 2 is evaluated as 1/x, 1, sqrt(x), x
 * or x*x (as NumPy's array ** scalar does); others by pow. */
#define FO_RATE_ARRHENIUS 0
#define FO_RATE_TROE 1
#define FO_RATE_USER 2
#define FO_RATE_SURFACE 3

typedef struct {
  int32_t type;     /* FO_RATE_* */
  int32_t column;   /* parameter column of FO_RATE_USER and FO_RATE_SURFACE, else -1 */
  double c[8];      /* the law's constants, as above */
} fo_rate_law;

/* k[c, j] for R reactions and C cells: laws (R, device), T and P (C, device),
 * params (device, column p of cell c at params[p * param_column_stride + c];
 * may be NULL when no law reads a column), power (R, device; the third-body
 * exponent, k *= M^power as fastode/ts1.py:100-102; NULL: none). The whole
 * TS1 rate-constant builder on the device. Asynchronous on stream. */
int fo_rate_laws(int32_t C, int32_t R, const fo_rate_law* laws, const double* T, const double* P,
                 const double* params, int64_t param_column_stride, const double* power, double* k,
                 int64_t k_cell_stride, int64_t k_reaction_stride, void* stream);

/* Photolysis columns at an interval start from per-cell factors the caller
 * computed: k[c, rxn[p]] = J[p] * f[c], one correctly rounded product, which
 * is the assignment k[:, photo] = J[None, photo] * f[:, None] of a host rate
 * constant builder (the per-interval photolysis patch of
 * fastode/ts1.py:204-214 with the diurnal factor evaluated by the caller).
 * Device pointers; asynchronous on stream. */
int fo_photolysis_factor(int32_t C, int32_t nphoto, const int32_t* rxn, const double* J, const double* f,
                         double* k, int64_t k_cell_stride, int64_t k_reaction_stride, void* stream);

/* Photolysis columns of one interval of a TS1 scenario:
 * k(c, rxn[p]) = (base[p * C + c] * factor) * scaling[p], the per-interval
 * patch of fastode/ts1.py:204-214 (run_scenario sets params[name] = base * f
 * and then k[:, j] = params[name] * scaling factor). rxn, base (nphoto x C,
 * cells fastest), scaling (nphoto) and k are device pointers; asynchronous. */
int fo_scale_photolysis(int32_t C, int32_t nphoto, const int32_t* rxn, const double* base, const double* scaling,
                        double factor, double* k, int64_t k_cell_stride, int64_t k_reaction_stride, void* stream);

/* Sample rules of the accuracy score. TS1 is fastode.ts1.score
 * (fastode/ts1.py:252-253): a sample is skipped when ref < threshold (a NaN
 * reference is counted). DIGITS is fastode.reference.digits
 * (fastode/reference.py:49): a sample is kept when ref >= threshold. */
#define FO_SCORE_TS1 0
#define FO_SCORE_DIGITS 1

/*
 * The sums behind Sandu's digits (fastode/ts1.py:226-264,
 * fastode/reference.py:41-59) for one snapshot of C cells, accumulated into
 * device arrays: for every reference column j with species[j] >= 0 and every
 * cell c whose reference value r = ref(c, j) is a sample under `rule`,
 *     sums[j] += ((Y(c, species[j]) - r) / r)^2,   counts[j] += 1.
 * Digits are then min(16, -log10(sqrt(sum / count))) per column and over all
 * columns (16 when the mean is <= 0). When gate is not NULL it is set to 0 if
 * any of the n species of any cell of Y is non-finite or below -1e-20
 * (fastode/ts1.py:240-241); it is never set to 1, so start it at 1.
 * Element (c, s) of Y is Y[c * y_cell_stride + s * y_species_stride] and
 * element (c, j) of ref is ref[c * ref_cell_stride + j * ref_column_stride].
 * species (m), ref, sums (m), counts (m), gate: device. Each column is
 * reduced by one block in a fixed order: the sums are reproducible bit for
 * bit. Asynchronous on `stream`.
 */
int fo_score_accumulate(int32_t C, int32_t n, const double* Y, int64_t y_cell_stride, int64_t y_species_stride,
                        int32_t m, const int32_t* species, const double* ref, int64_t ref_cell_stride,
                        int64_t ref_column_stride, double threshold, int32_t rule, double* sums, int64_t* counts,
                        int32_t* gate, void* stream);

/* FP64 fused multiply-add throughput of the current device (FMA per second),
 * measured with a full-warp DFMA kernel: the roofline denominator for the
 * integrator. No counterpart in the reference (which never times work). */
int fo_fp64_fma_rate(double* fma_per_second);

/* Bytes of the static device scratch of fo_solve_static. */
#define FO_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)

/*
 * fo_solve without a workspace and without any device allocation. No
 * counterpart in the reference: it exists for callers that cannot allocate
 * device memory while they integrate — a host model that gives the device to
 * its own memory pool at start-up and forbids allocations afterwards, or a
 * time step that cannot afford the implicit device synchronization of
 * cudaMalloc/cudaFree. The caller still passes every input and output (same
 * meaning as fo_solve); the scratch is one file-scope device array of
 * FO_STATIC_SCRATCH_BYTES (32 MiB) that every GPU loading the library holds
 * until the process exits, holding as many groups in flight as fit: one slot
 * per group in flight, of fo_workspace_bytes(plan, 2, C) -
 * fo_workspace_bytes(plan, 1, C) bytes (a 210-species / 500-reaction group of
 * 32 cells needs about 4.2 MB, so seven at a time); more groups than slots are
 * pulled from a device queue by the slots in turn. A mechanism whose single
 * group does not fit is rejected with FO_E_UNSUPPORTED. The first call on each
 * device looks up the array's device address and should come before any stream
 * capture; the address is kept for the life of the process, so after
 * cudaDeviceReset (or anything else that destroys the device's primary
 * context) this entry point must not be called again in that process. All
 * calls share the array: calls whose kernels overlap on the GPU race on it, so
 * order them on one stream.
 */
int fo_solve_static(const fo_plan* plan, const fo_options* opt, int32_t ngroups, const int32_t* group_offsets,
                    int32_t max_group_cells, double* Y, int64_t y_cell_stride, int64_t y_species_stride,
                    const double* k, int64_t k_cell_stride, int64_t k_reaction_stride, const double* atol,
                    double rtol, double dt, double* memory, int64_t* counts, int32_t* status, void* stream);

/* Last CUDA error text seen by the library (thread-local, never NULL). */
const char* fo_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* FASTODE_GB300_H */
