/*
 * gridoxide_gb300.h -- C ABI of the GB300 batched Newton-Raphson power-flow
 * engine.  Plain pointers and sizes only; link against
 * libgridoxide_gb300.so.
 *
 * Two levels, mirroring the reference's plugin surface:
 *
 *  1. gox_ls_*    -- one sparse system, the solver::LinearSolver trait
 *                    (gridoxide src/solver.rs:35-57) that KluNativeSystem
 *                    implements (src/klu_native/mod.rs:136-211).
 *  2. gox_topo_* / gox_batch_* -- one topology, many scenarios: what
 *                    batch::BatchSolver::solve does (src/batch.rs:198-289)
 *                    with PersistentSolver's cached pattern and pivot order
 *                    (src/solver.rs:395-494), run on the GPU.
 *
 * Status convention: 0 = OK; GOX_SINGULAR (1) = structurally or numerically
 * singular (the trait's `None`); negative = error (KLU_INVALID /
 * KLU_OUT_OF_MEMORY / BatchError analogues below).  Handles are not
 * thread-safe: use one per host thread, like the reference's !Send FFI
 * backends (src/batch.rs:234-246).
 *
 * All host buffers are caller-owned.  Per-scenario arrays are row-major
 * [scenario][bus].  Bus types: 1 PQ, 2 PV, 3 slack (src/types.rs:26-42).
 */
#ifndef GRIDOXIDE_GB300_H
#define GRIDOXIDE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GOX_OK 0
#define GOX_SINGULAR 1          /* LinearSolver returned None (KLU_SINGULAR) */
#define GOX_PENDING 2           /* gox_server_poll: the request is not solved yet */
#define GOX_E_OUT_OF_MEMORY (-2) /* KLU_OUT_OF_MEMORY */
#define GOX_E_INVALID (-3)      /* KLU_INVALID: bad sizes / pointers / pattern */
#define GOX_E_BUS_RANGE (-4)    /* BatchError::BusOutOfRange (src/batch.rs:108-135) */
#define GOX_E_CUDA (-5)         /* a CUDA runtime call failed */
#define GOX_E_PATTERN (-6)      /* values given for a different pattern */
#define GOX_E_NO_DEVICE (-7)    /* no CUDA device visible */
#define GOX_E_TOO_LARGE (-8)    /* request exceeds a documented size limit */
#define GOX_E_DEVICE_WAIT (-9)  /* a bounded wait inside a kernel gave up; results invalid */

/* per-scenario outcome, solver::SolveStatus (src/solver.rs:162-171) */
#define GOX_CONVERGED 0
#define GOX_MAX_ITERATIONS 1
#define GOX_SINGULAR_SCENARIO 2

/* arithmetic of the Jacobian refactorization and triangular solves; the
 * mismatch, convergence test and voltage update are always FP64 */
#define GOX_PRECISION_FP64 0
#define GOX_PRECISION_MIXED 1   /* FP32 refactor/solve, FP64 mismatch */

/* ---- level 1: LinearSolver ------------------------------------------- */
typedef struct gox_ls gox_ls;

/* LinearSolver::new (src/solver.rs:38-41; KluNativeSystem::new,
 * src/klu_native/mod.rs:159-169): analyze the (row, col) pattern (BTF + AMD),
 * factor `vals` once with partial pivoting (tol 0.001) to fix the pivot
 * order.  Duplicate (row, col) entries are summed.  *out = NULL and
 * GOX_SINGULAR if the matrix is singular. */
int gox_ls_create(int32_t n, int32_t nnz, const int32_t *rows, const int32_t *cols,
                  const double *vals, gox_ls **out);

/* LinearSolver::factor_and_solve_values (src/solver.rs:56;
 * src/klu_native/mod.rs:208-210): refactor on the GPU with the fixed pivot
 * order (FP64) and solve A x = rhs.  vals positionally match the triplets
 * given to gox_ls_create.  GOX_SINGULAR on a zero pivot or non-finite x. */
int gox_ls_factor_solve_values(gox_ls *h, const double *vals, const double *rhs, double *x);

/* LinearSolver::factor_and_solve (src/solver.rs:44-45): as above, but the
 * caller passes the triplets again; they must equal those given to
 * gox_ls_create, position by position (GOX_E_PATTERN otherwise). */
int gox_ls_factor_solve(gox_ls *h, int32_t nnz, const int32_t *rows, const int32_t *cols,
                        const double *vals, const double *rhs, double *x);

/* Drop (src/sparse_klu.rs:205-212). */
void gox_ls_destroy(gox_ls *h);

/* No counterpart in the reference.  gox_ls_factor_solve_values for callers
 * that cannot allocate device memory at solve time: a process whose device
 * memory was handed up front to another allocator (a framework's caching
 * pool, a serving process that reserves HBM at start-up), where cudaMalloc
 * fails or takes memory the pool counted on; and a control loop with a
 * deadline per Newton step, where cudaMalloc / cudaFree synchronize the
 * device and take unbounded time.  The refactor and solve use no device
 * buffer of the handle: their scratch (the factor values, right-hand side,
 * solution and flags) lives in one fixed array compiled into the library,
 * GOX_STATIC_SCRATCH_BYTES per device, held by every process that loads the
 * library until it exits.  Nothing is allocated or freed on the device by
 * this call.
 *   - Limit: 32 * 8 * (LU slots + off-diagonal entries + 2 n) plus
 *     12 * nnz + 16 * n bytes must fit in GOX_STATIC_SCRATCH_BYTES
 *     (GOX_E_TOO_LARGE otherwise; about 260k factor entries).
 *   - The first call on a device looks up the array's device address
 *     (cudaGetSymbolAddress) with that device current and keeps it for the
 *     process; make that first call before any stream capture.  The address
 *     belongs to the device's CUDA context: after cudaDeviceReset the
 *     process must not call this entry again.
 *   - All calls share the one array and leave the last call's values in
 *     it; calls that overlap on the GPU (other host threads, other handles)
 *     overwrite each other's scratch: serialize them.
 * Same arguments and results as gox_ls_factor_solve_values. */
#define GOX_STATIC_SCRATCH_BYTES (64u << 20)
int gox_ls_factor_solve_values_static(gox_ls *h, const double *vals, const double *rhs,
                                      double *x);

/* ---- level 2: batched Newton-Raphson --------------------------------- */
typedef struct gox_topo gox_topo;

/* Registers a topology: the frozen Y-bus in CSR form (each row's columns
 * ascending, duplicates already summed -- YBus::finish, src/network.rs:52-71)
 * and the bus types.  Computes the Jacobian pattern
 * (JacobianPattern::analyze, src/jacobian.rs:96-171) and its symbolic
 * ordering (klu_native analyze, src/klu_native/analyze.rs:67-150).  The
 * numeric pivot order is fixed later by the first Jacobian factored, as in
 * PersistentSolver. */
int gox_topo_register(int32_t n_bus, const int32_t *y_rowptr, const int32_t *y_col,
                      const double *y_re, const double *y_im, const int32_t *bus_type,
                      gox_topo **out);

/* PersistentSolver::reset (src/solver.rs:480-493): forget the pivot order
 * (the next solve refactors from a fresh partial-pivoting factorization). */
int gox_topo_reset(gox_topo *t);

void gox_topo_destroy(gox_topo *t);

/* BatchSolver::solve on the GPU.  B scenarios of one topology.
 *   p_spec, q_spec [B][n_bus]: net injections (BusOverride p/q already
 *       applied; src/batch.rs:254-266);
 *   vm0, va0: start voltages, [B][n_bus] when v_stride == n_bus or one
 *       shared [n_bus] template when v_stride == 0.  Slack and PV entries
 *       of vm0 are the voltage set-points;
 *   out_slot, out_dre, out_dim [B][4] or NULL: per-scenario Y-bus deltas
 *       (N-1 branch outage with the pattern kept): the four slots of the
 *       branch's (ff, ft, tf, tt) entries and the values added to them;
 *       out_slot[4s] < 0 means no outage for scenario s;
 *   tol, max_iter: newton_raphson_cached's strict `max|F| < tol` and
 *       iteration cap (src/solver.rs:699-703);
 *   precision: GOX_PRECISION_FP64 or GOX_PRECISION_MIXED;
 *   outputs: vm/va [B][n_bus], iterations (= mismatch-history length),
 *       status (GOX_CONVERGED ...), final max mismatch [B], history
 *       [B][max_iter] or NULL.
 * Non-convergence is not an error (src/batch.rs:193-197).  Returns
 * GOX_E_BUS_RANGE if an outage slot is outside the Y-bus. */
int gox_batch_solve(gox_topo *t, int32_t B, const double *p_spec, const double *q_spec,
                    const double *vm0, const double *va0, int32_t v_stride,
                    const int32_t *out_slot, const double *out_dre, const double *out_dim,
                    double tol, int32_t max_iter, int32_t precision, double *vm_out,
                    double *va_out, int32_t *iterations, int32_t *status, double *max_mismatch,
                    double *history);

/* As gox_batch_solve, with every array in device memory and the work
 * enqueued on `stream` (a cudaStream_t, NULL = legacy default stream).
 * Synchronizes with the stream once per Newton iteration to read the
 * running-scenario count. */
int gox_batch_solve_device(gox_topo *t, int32_t B, const double *p_spec, const double *q_spec,
                           const double *vm0, const double *va0, int32_t v_stride,
                           const int32_t *out_slot, const double *out_dre,
                           const double *out_dim, double tol, int32_t max_iter,
                           int32_t precision, double *vm_out, double *va_out,
                           int32_t *iterations, int32_t *status, double *max_mismatch,
                           double *history, void *stream);

/* gox_batch_solve for the time-series / Monte Carlo shape: scenario s has
 * p_spec = p_base * scales[s] and q_spec = q_base * scales[s] (host arrays
 * p_base, q_base [n_bus], scales [B]; vm0/va0 [n_bus] shared).  Replaces
 * `BatchSolver::solve` over `uniform_load_scaling` scenarios
 * (src/batch.rs:98-106, the reference model's `solve_batch_scaled`,
 * src/python.rs:323-343): the scenarios are expanded on the device, so only
 * n_bus + B values cross to it.  Outputs as gox_batch_solve. */
int gox_batch_solve_scaled(gox_topo *t, int32_t B, const double *scales, const double *p_base,
                           const double *q_base, const double *vm0, const double *va0,
                           double tol, int32_t max_iter, int32_t precision, double *vm_out,
                           double *va_out, int32_t *iterations, int32_t *status,
                           double *max_mismatch, double *history);

/* Many topologies' batches solved together: the reference's BatchSolver
 * work queue over scenarios of uneven cost (src/batch.rs:230-281), here for
 * n_topo topologies at once.  By default one Newton loop runs each phase
 * as one launch over every topology still running (update, injections,
 * decision, fill, one launch per wide level, the refactor's CTAs largest
 * topology first); a topology leaves the loop when its last scenario has
 * converged or failed.  With gox_set_multi_persistent(1) one persistent
 * kernel launch solves everything instead: each CTA takes (topology, group
 * of 32 scenarios) items from a device-side queue, largest topology first,
 * and runs that group's whole Newton loop, each topology on a refactor plan
 * without the wide split (compiled once; a topology whose BTF form has
 * off-diagonal blocks, or for which no such plan fits, sends the call to
 * the loop).  Each topology's set-up and results run on up to 8 host
 * threads.  Per topology j the arguments are gox_batch_solve's: batch[j]
 * scenarios, p_spec[j] / q_spec[j] [batch[j]][n_bus], vm0[j] / va0[j] with
 * v_stride[j], outputs vm_out[j], va_out[j], iterations[j], status[j],
 * max_mismatch[j] (host arrays); tol, max_iter and precision are shared.
 * The results equal gox_batch_solve's on each topology alone, bit for bit.
 * No outages and no ZIP terms (GOX_E_INVALID), each topology at most once,
 * max_iter >= 1. */
int gox_set_multi_persistent(int32_t on);
int gox_multi_solve(int32_t n_topo, gox_topo *const *topos, const int32_t *batch,
                    const double *const *p_spec, const double *const *q_spec,
                    const double *const *vm0, const double *const *va0, const int32_t *v_stride,
                    double tol, int32_t max_iter, int32_t precision, double *const *vm_out,
                    double *const *va_out, int32_t *const *iterations, int32_t *const *status,
                    double *const *max_mismatch);

/* Batched solve with reactive-power limits on the PV buses: per scenario
 * the reference's newton_raphson_enforcing_q_limits (src/solver.rs:545-618).
 * After a converged solve, every PV bus whose computed Q lies outside
 * [q_min[b], q_max[b]] (per unit, arrays [n_bus]; -inf/+inf for none)
 * becomes PQ with q_spec pinned at the violated limit, and the scenario is
 * solved again from its converged state; repeated until no bus switches
 * (stabilized = 1) or max_outer solves have run (stabilized = 0, the last
 * solve's report).  A scenario whose solve did not converge stops with that
 * report.  Switching is one-way.  Scenarios with the same switched set are
 * solved together on a cached variant of the topology with those bus types.
 * iterations / status / max_mismatch describe the last solve; n_switched [B]
 * counts the switched buses and `switched` ([B][n_bus] bytes, or NULL)
 * marks them.  Inputs and outputs are host arrays as in gox_batch_solve. */
int gox_batch_solve_qlim(gox_topo *t, int32_t B, const double *p_spec, const double *q_spec,
                         const double *vm0, const double *va0, int32_t v_stride,
                         const double *q_min, const double *q_max, double tol, int32_t max_iter,
                         int32_t max_outer, int32_t precision, double *vm_out, double *va_out,
                         int32_t *iterations, int32_t *status, double *max_mismatch,
                         int32_t *n_switched, uint8_t *switched, int32_t *stabilized);

/* Islands of outage scenarios (network::connected_components / classify,
 * src/network.rs:121-194).  An outage whose off-diagonal Y entries become
 * exactly zero removes its branch from the graph; when that branch is a
 * bridge the grid splits.  The batched solves (gox_batch_solve,
 * gox_batch_solve_device, the server) pin every component without a slack
 * bus to V = 0 with no injection (mark_unreferenced_islands,
 * src/network.rs:196-223) and solve the rest, so such a scenario reports
 * Converged for its energized part.  This call describes the split without
 * solving: per scenario the number of components (n_islands [B]), each bus's
 * component in connected_components order (island_of [B][n_bus] or NULL)
 * and its component's verdict (verdict [B][n_bus] or NULL, classify's
 * Verdict: one slack bus, none, or several).  Host arrays, no GPU needed. */
#define GOX_ISLAND_SOLVABLE 0
#define GOX_ISLAND_NO_REFERENCE 1
#define GOX_ISLAND_AMBIGUOUS 2
int gox_outage_islands(gox_topo *t, int32_t B, const int32_t *out_slot, const double *out_dre,
                       const double *out_dim, int32_t *n_islands, int32_t *island_of,
                       int32_t *verdict);

/* Fixes the topology's pivot order on the host, without a GPU: the first
 * scenario whose start point misses `tol` has its Jacobian factored with
 * partial pivoting (KluNativeSystem::new on the first Jacobian a
 * PersistentSolver sees, src/solver.rs:711-713).  Arguments as for
 * gox_batch_solve.  A later gox_batch_solve* reuses this order.  Returns
 * GOX_SINGULAR if no scenario's Jacobian factors. */
int gox_topo_prepare(gox_topo *t, int32_t B, const double *p_spec, const double *q_spec,
                     const double *vm0, const double *va0, int32_t v_stride,
                     const int32_t *out_slot, const double *out_dre, const double *out_dim,
                     double tol);

/* Host mirror of the device refactor + substitution schedule for one
 * scenario, in FP64: Jacobian values in emission order, right-hand side in
 * unknown order, solution dx in unknown order.  Needs a fixed pivot order.
 * Returns GOX_SINGULAR on a zero pivot or non-finite dx. */
int gox_topo_emulate_step(const gox_topo *t, const double *jac_vals, const double *rhs,
                          double *dx);

/* ---- inspection (klu_analyze / klu_extract analogues) ------------------ */

/* The device path's Jacobian and factor values at given voltages (the
 * per-entry view of JacobianPattern::fill, src/jacobian.rs:202-250, and of
 * the refactor, src/klu_native/refactor.rs:68-152, that klu_extract gives
 * for KLU): for B scenarios (host arrays p_spec, q_spec, vm, va
 * [B][n_bus]) one injection + mismatch, one Jacobian fill and one refactor
 * with the fixed pivot order run on the GPU in `precision`.  jac_vals
 * [B][nnz J] (emission order, or NULL) receives the filled Jacobian;
 * lu_vals [B][LU slots] (or NULL) the factor, column by column in factor
 * order: the column's U entries (gox_topo_structure's Ui order), its
 * diagonal, then its L entries (Li order, divided by the pivot).  Needs a
 * fixed pivot order. */
int gox_topo_factor_values(gox_topo *t, int32_t B, const double *p_spec, const double *q_spec,
                           const double *vm, const double *va, int32_t precision,
                           double *jac_vals, double *lu_vals);

/* The mixed path's repair of a poor static pivot order, on one Jacobian:
 * the FP64 threshold-partial-pivoting factorization the GPU runs for the
 * Newton steps of scenarios that trip the pivot-ratio check (Gilbert-Peierls
 * per BTF block with KLU's lpivot, tol 0.001 and diagonal preference --
 * src/klu_native/kernel.rs:187-262, 341-416 -- pivots chosen afresh for
 * these values, then the block substitutions of src/klu_native/solve.rs:
 * 56-102).  jac_vals in emission order, rhs and dx in unknown order.  Needs
 * a fixed (static) pivot order, which only lays out the inputs.  Returns
 * GOX_SINGULAR on a zero pivot, a factor above its fill bound (three times
 * the static factor plus 4 n entries) or a non-finite dx. */
int gox_topo_pivot_solve(gox_topo *t, const double *jac_vals, const double *rhs, double *dx);

/* Test hook, no counterpart in the reference: replaces word `index` of warp
 * `warp`'s refactor command stream (FP32 plan for GOX_PRECISION_MIXED, FP64
 * plan otherwise) on the device with `value` and returns the old word, so a
 * test can plant a malformed command and restore the stream.  A refactor
 * that meets a malformed command stops that warp, drains its copies, keeps
 * the CTA's barriers and makes the solve return GOX_E_DEVICE_WAIT.  The
 * stream must have been uploaded (a solve ran). */
int gox_topo_stream_word(gox_topo *t, int32_t precision, int32_t warp, int32_t index,
                         int32_t value, int32_t *old_value);

/* klu_analyze on a CSC pattern (BTF + AMD): P, Q [n], R [n+1]; returns the
 * number of blocks or < 0. */
int gox_analyze(int32_t n, const int32_t *Ap, const int32_t *Ai, int32_t *P, int32_t *Q,
                int32_t *R);

/* klu_analyze + klu_factor + klu_extract analogue on the host, no GPU:
 * the partial-pivoting factorization whose pivot order the GPU refactor
 * reuses (KluNativeSystem::new, src/klu_native/mod.rs:159-169).  Triplets
 * as for gox_ls_create.  sizes[0] = nnz L incl. unit diagonal, [1] = nnz U
 * incl. diagonal, [2] = nnz off-diagonal, [3] = nblocks.  With Lp == NULL
 * only sizes are written.  Layout of klu_extract: L columns start with the
 * unit diagonal, U columns end with the diagonal, rows in pivot order; P is
 * the final row permutation (Pnum).  Returns GOX_SINGULAR if singular. */
int gox_factor_host(int32_t n, int32_t nnz, const int32_t *rows, const int32_t *cols,
                    const double *vals, int64_t *sizes, int32_t *Lp, int32_t *Li, double *Lx,
                    int32_t *Up, int32_t *Ui, double *Ux, int32_t *Fp, int32_t *Fi, double *Fx,
                    int32_t *P, int32_t *Q, int32_t *R);

/* Sizes of the topology's Jacobian and factor, once its pivot order is
 * fixed: [0] n unknowns, [1] nnz J, [2] nnz L (no diag), [3] nnz U (no
 * diag), [4] nnz off-diagonal, [5] BTF blocks, [6] refactor levels,
 * [7] solve phases, [8] LU slots per scenario, [9] max column length;
 * refactor schedule of the FP32 plan: [10] warps per CTA, [11] ring rows
 * per warp, [12] estimated critical path (cycles), [13] rows read in place
 * from another column's shared-memory block, [14] rows copied from global
 * memory, [15] of them issued a column ahead, [16] issued at the column's
 * start, [17] issued just in time, [18] update steps, [19] waits; the FP64
 * plan: [20] warps, [21] ring rows, [22] estimated cycles, [23] rows read
 * in place; [24] columns of the FP32 plan run as one command, [25] its
 * stream words; [26] / [27] 1 when the FP32 / FP64 refactor also runs the
 * backward substitution (no separate solve launch); [28] columns of the FP32
 * plan whose update prefix runs one level early; [29] rows of the FP32 plan
 * copied by warps idle in a level for another warp's next column; [30]
 * solves of this topology whose Newton loop ran as one captured CUDA graph
 * (a configuration seen before: same batch buffers, precision, budget);
 * [31] 1 when the FP32 plan's levels end in per-warp progress flags (0: CTA
 * barriers), [32] its progress-flag wait commands, [33] the warps those
 * commands wait for, summed; [34] / [35] refactor levels / backward phases
 * of the FP32 plan the wide kernels run.  info must hold 36 entries.
 * Returns GOX_E_INVALID before the first solve. */
int gox_topo_info(const gox_topo *t, int64_t *info);

/* The refactor plan's autotuner (no counterpart in the reference: its KLU
 * runs one fixed kernel; the nearest knobs are KLU's fixed Options,
 * src/klu_native/types.rs:73-99).  A topology's first batch in a precision
 * times the candidate plans of its refactor streams -- warps per CTA (12
 * down to 4 in FP32, 8 down to 4 in FP64) x stream chunks of 256 / 320 /
 * 512 words x the levels' synchronization (per-warp progress flags or CTA
 * barriers) x without / with the wide kernels (gox_set_refactor_wide),
 * each compiled and checked on the host first -- on the first
 * min(G, 152) groups of that batch's first Jacobian (CUDA events, two runs
 * each) and keeps the fastest.  Choices are cached per process, and in the
 * file named by $GOX_TUNE_CACHE when set, under (precision, bus count in
 * half-octave buckets, fill nnz(L+U) / nnz(J) in tenths, batch-size bucket
 * of 1 / 2-8 / 9-38 / 39-152 / more groups of 32); a later topology with
 * the same key compiles the cached plan without timing.  Q-limit and
 * island variants take a cached plan or the default.  gox_set_autotune(0)
 * turns it off process-wide: the default plan is the most warps that fit,
 * with the levels' synchronization of gox_set_refactor_sync. */
int gox_set_autotune(int32_t on);

/* How the default refactor plan (the one used without the autotuner, and
 * before it has timed anything) ends each dependency level: flags = 1
 * per-warp progress flags -- each warp publishes the levels it has done
 * and waits only for the warps whose earlier work it reads or overwrites,
 * as found by the stream compiler --, 0 (default) CTA barriers.  Both
 * forms run the same operations in the same order per value, so the
 * results are bit-identical; the autotuner times both.  (Measured on
 * case2000 x 4,096, 12 warps: FP32 2.19 ms with barriers, 2.27 ms with
 * flags -- the critical path is the column chain itself, not the barrier
 * -- and FP64 7.71 / 7.60 ms at 7 warps.)  Applies to topologies analysed
 * afterwards.
 * (No counterpart in the reference: its KLU refactor is sequential per
 * scenario, src/klu_native/kernel.rs:476-524.) */
int gox_set_refactor_sync(int32_t flags);

/* The wide kernels in the default refactor plan: min_width > 0 hands the
 * leading refactor levels with at least min_width columns each (columns of
 * at most 128 entries), and afterwards the backward-substitution rows of
 * those columns (from the last such level down), to kernels that run one
 * level per launch with one warp per (column or row, group of 32
 * scenarios) across every SM; the per-group refactor kernel runs the rest.
 * 0 (default) keeps every level in the per-group kernel.  The results are
 * bit-identical either way; the autotuner times the plans without the
 * split and with it at min_width 64 and 16.
 * Applies to topologies analysed afterwards; GOX_E_INVALID for < 0.  (No
 * counterpart in the reference: KLU's refactor is one sequential sweep per
 * scenario, src/klu_native/kernel.rs:476-524, solve.rs:56-102.) */
int gox_set_refactor_wide(int32_t min_width);

/* The plan a topology's refactor runs in `precision`: plan[0] warps per
 * CTA, [1] ring rows per warp, [2] rows of warp 0's larger ring (0: none),
 * [3] stream-chunk words, [4] source (0 default, 1 timed by the autotuner,
 * 2 from its cache), [5] candidates timed, [6] 1 when the levels end in
 * per-warp progress flags, 0 in CTA barriers, [7] / [8] refactor levels /
 * backward phases the wide kernels run (plan must hold 9 entries).  With
 * `table`, up to max_rows rows {warps, chunk words, ring rows, ms,
 * progress flags, wide levels, wide phases} of the timed candidates;
 * returns the rows written, or < 0.  Needs a fixed pivot order. */
int gox_topo_tuning(const gox_topo *t, int32_t precision, int64_t *plan, double *table,
                    int32_t max_rows);

/* The fixed factorization structure (klu_extract layout without values):
 * Pnum, Q [n], R [nblocks+1], L pattern Lp [n+1] / Li (rows in pivot order,
 * no unit diagonal), U pattern Up [n+1] / Ui (DFS order, no diagonal).
 * Also the refactor flop count per scenario in flops[0] and the solve flop
 * count in flops[1]. */
int gox_topo_structure(const gox_topo *t, int32_t *Pnum, int32_t *Q, int32_t *R, int32_t *Lp,
                       int32_t *Li, int32_t *Up, int32_t *Ui, double *flops);

/* The Jacobian pattern in emission order: rows, cols [nnz J]. */
int gox_topo_jacobian_pattern(const gox_topo *t, int32_t *rows, int32_t *cols);

/* Timing of the last gox_batch_solve*: [0] iterations run, [1] total kernel
 * ms, [2] mismatch ms, [3] fill ms, [4] refactor ms, [5] solve ms (CUDA
 * events on the solve stream; only when timing was enabled). */
int gox_set_timing(gox_topo *t, int32_t enable);
int gox_last_timing(const gox_topo *t, double *out);

/* Kernel launches issued by the last gox_batch_solve* call. */
int64_t gox_last_launches(const gox_topo *t);
/* Re-packs so far by this topology's solves (its split parts' included):
 * in the host-driven Newton loop, once the scenarios still running fit in at
 * most half of the groups still active (16 or more), they move into the
 * first lanes of a smaller batch for the remaining iterations and their
 * results back at the end -- the same results bit for bit, fewer groups for
 * the mismatch, fill and refactor launches.  A configuration whose solve
 * re-packed stays on the host-driven loop (no captured graph). */
int64_t gox_topo_repacks(const gox_topo *t);
/* Re-packing on (1, the default) or off (0), process-wide. */
int gox_set_repack(int32_t on);

/* Start point of the batched solves.  GOX_GUESS_GIVEN (default): the
 * vm0/va0 passed to the call.  GOX_GUESS_LINEAR: the reference BatchSolver's
 * linear initial guess (src/batch.rs:268 -> linear_initial_guess,
 * src/network.rs:627-678) computed from them on the GPU: the PQ buses'
 * voltages solve Y'_nn U_n = -Y'_ns U_s, where Y' adds -conj(p + jq) to the
 * diagonal of every PQ bus and U_s are the given voltages of the other buses
 * (a scenario whose system is singular keeps its given start).  The complex
 * system is solved as its real 2x2-block form, refactored in FP64 with the
 * pivot order of its first factorization (the reference's faer complex LU,
 * src/sparse.rs:48-63, pivots per call; the results agree to rounding).
 * With an outage the guess uses the scenario's modified Y-bus. */
/* ZIP terms of the effective injection (src/network.rs:600-611): per bus a
 * constant-impedance and a constant-current complex injection (per unit at
 * |V| = 1, each the sum of that bus's terms of the kind), added to the
 * scenario's p_spec + j q_spec as s_imp |V| |V| + s_cur |V| at the present
 * |V| in every mismatch (and in the linear initial guess).  As in the
 * reference they are not differentiated in the Jacobian (src/jacobian.rs:
 * 224-243 uses only the computed injections).  Arrays [n_bus]; all four
 * NULL clears them. */
int gox_topo_set_zip(gox_topo *t, const double *zi_re, const double *zi_im, const double *zc_re,
                     const double *zc_im);

/* Newton loop as a captured CUDA graph (default on): from the second solve
 * of a configuration (same batch buffers, precision, budget, outage use)
 * the whole loop is one graph launch with conditional while / if nodes and
 * the iteration on the device, instead of host-driven launches with one
 * synchronization per iteration; results are the same bit for bit.  Only
 * batches of at least 2,048 scenarios use it (smaller ones measured slower
 * as graphs when many topologies solve concurrently).  0 keeps this
 * topology on the host-driven loop. */
int gox_topo_set_graph(gox_topo *t, int32_t on);

/* Split solves (parts 1..8, or 0, the default: two parts, four from 8,192
 * scenarios): once the pivot order is fixed, a mixed-precision batch of
 * 4,096+ scenarios with the given start is solved as `parts` parts of whole
 * groups of 32 scenarios at the same time, part k
 * by the k-th instance of the topology (a chain of clones) on its own stream
 * from its own host thread, started k fractions of an iteration later so
 * that one part's mismatch and fill overlap the others' refactors.  Every
 * result is the same as unsplit, bit for bit. */
int gox_topo_set_split(gox_topo *t, int32_t parts);

#define GOX_GUESS_GIVEN 0
#define GOX_GUESS_LINEAR 1
int gox_topo_set_initial_guess(gox_topo *t, int32_t mode);

/* The linear initial guess itself (what the GOX_GUESS_LINEAR mode starts
 * Newton from), computed on the GPU for B scenarios: host arrays p_spec,
 * q_spec [B][n_bus], vm0/va0 [n_bus] (v_stride 0) or [B][n_bus] (v_stride
 * n_bus); vm_out/va_out [B][n_bus].  Replaces the reference model's
 * `initial_guess()` (src/python.rs:395-406, one scenario).  When the guess
 * system is singular at its first factorization the given start is
 * returned. */
int gox_topo_initial_guess(gox_topo *t, int32_t B, const double *p_spec, const double *q_spec,
                           const double *vm0, const double *va0, int32_t v_stride,
                           double *vm_out, double *va_out);

/* Mixed path: the pivot-ratio threshold.  A scenario whose FP32 refactor
 * meets a pivot with |u_kk| < tol * max |L(:, k)| (before scaling) is solved
 * again from its start point on the FP64 path, each of its Newton steps
 * factoring its Jacobian with threshold partial pivoting on the GPU
 * (KLU_factor's pivoting, src/klu_native/kernel.rs:187-262, 341-416; see
 * gox_topo_pivot_solve), and that report replaces its mixed one.  Default
 * 1e-6; 0 disables.  No counterpart in the reference (its refactor is FP64
 * only and keeps its pivots). */
int gox_set_pivot_tolerance(gox_topo *t, double tol);

/* Scenarios of the last gox_batch_solve / gox_batch_solve_device call that
 * were solved again in FP64 (see gox_set_pivot_tolerance). */
int64_t gox_last_fallbacks(const gox_topo *t);

/* Library version string. */
const char *gox_version(void);

/* ---- serving --------------------------------------------------------------
 * Continuous batching of single-scenario requests over registered
 * topologies: each of 16 worker threads takes the oldest queued request
 * whose topology has a free lane and up to max_batch of that topology's
 * requests (arrival order), solves them with gox_batch_solve on its own
 * stream (batches of different topologies, and of one topology on its
 * lanes, overlap on the GPU), and publishes each result with its latency
 * (submit to completion).  A topology's lanes are the topology itself and,
 * after its first batch has fixed its pivot order and plan, clones of it
 * with their own device state (gox_server_set_lanes); every lane gives the
 * same results bit for bit.  Scenarios are independent, so a request's
 * result does not depend on the batch it ran in.  A topology added to a server is used by the server's workers
 * only: do not call it directly while the server runs.  Its refactor plan
 * is timed by the autotuner on its first batch at most; later batches keep
 * that plan (or a cached one), so no timing runs inside the serving loop.
 * The reference's serving counterpart is the Python `PowerFlowModel.solve_batch`
 * / rayon `BatchSolver` call per batch (src/python.rs:306-341,
 * src/batch.rs:198-289); the queue in front of it is new here. */
typedef struct gox_server gox_server;

int gox_server_create(int32_t max_batch, int32_t precision, double tol, int32_t max_iter,
                      gox_server **out);
/* Registers a topology (not owned by the server); its id in *topo_id. */
int gox_server_add_topology(gox_server *s, gox_topo *t, int32_t *topo_id);
/* Queues one scenario: p_spec, q_spec, vm0, va0 [n_bus]; optional outage
 * (4 Y slots and the values added to them, as gox_batch_solve's out_*;
 * all three or none).  Returns a ticket. */
int gox_server_submit(gox_server *s, int32_t topo_id, const double *p_spec, const double *q_spec,
                      const double *vm0, const double *va0, const int32_t *out_slot,
                      const double *out_dre, const double *out_dim, int64_t *ticket);
/* Queues `count` requests in one call, each as gox_server_submit would
 * (request k: topo_ids[k], p_spec[k], q_spec[k], vm0[k], va0[k] [n_bus of
 * its topology]; out_slot / out_dre / out_dim NULL for no outages, else
 * arrays of count pointers, NULL for a request without one), all with the
 * same submit time; their tickets in tickets[count].  Every request is
 * checked first: GOX_E_INVALID queues none.  A front end that drains its
 * receive queue periodically submits what arrived at once. */
int gox_server_submit_many(gox_server *s, int32_t count, const int32_t *topo_ids,
                           const double *const *p_spec, const double *const *q_spec,
                           const double *const *vm0, const double *const *va0,
                           const int32_t *const *out_slot, const double *const *out_dre,
                           const double *const *out_dim, int64_t *tickets);
/* GOX_PENDING until the request is solved; then GOX_OK (the outputs are
 * written and the ticket is retired) or the batch's error code.  Output
 * pointers may be NULL. */
int gox_server_poll(gox_server *s, int64_t ticket, double *vm, double *va, int32_t *iterations,
                    int32_t *status, double *max_mismatch, double *latency_s);
/* out[8]: [0] batches run, [1] requests solved, [2] requests queued, [3]
 * device bytes the topologies' batch buffers hold now, [4] their peak, [5] /
 * [6] microseconds summed over the solved requests spent queued / in their
 * batch's solve, [7] topology clones made for lanes. */
int gox_server_stats(gox_server *s, int64_t *out);
/* Lanes per topology, 1..8 (default 1): how many batches of one topology
 * may be solved at the same time.  Lanes beyond the first are clones made
 * on first use (host copies of the topology's analysis and plans, device
 * buffers of their own); with an HBM budget set, one lane per topology. */
int gox_server_set_lanes(gox_server *s, int32_t lanes);
/* Admission by HBM budget (bytes; 0, the default: none).  A worker admits
 * at most the batch whose buffers fit in the budget beside the other
 * topologies' buffers (by each topology's per-scenario device bytes),
 * releasing the buffers of idle topologies first when they do not; one
 * request is always admitted. */
int gox_server_set_budget(gox_server *s, int64_t bytes);
/* Finishes the queued requests, stops the worker, frees the server. */
void gox_server_destroy(gox_server *s);

#ifdef __cplusplus
}
#endif
#endif
