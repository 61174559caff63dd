/*
 * gox_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C CPU restatement of gridoxide's batched Newton-Raphson power-flow
 * path, used as the checker for the GPU engine and as the timed CPU
 * baseline.  Nothing in the product library includes, links or calls this.
 *
 *   Y-bus stamping        gridoxide src/network.rs:225-247, 339-373
 *   power_injections      src/network.rs:680-701 (+ faer SpMV, src/sparse.rs:32-36)
 *   effective_injection   src/network.rs:600-611 (constant power + ZIP terms)
 *   JacobianPattern       src/jacobian.rs:96-171 (analyze), 202-250 (fill)
 *   build_csc_structure   src/klu_native/mod.rs:88-125
 *   KLU numeric factor    src/klu_native/factor.rs:47-131, kernel.rs:32-416
 *                         (C original: KLU/Source/klu_kernel.c, klu_factor.c)
 *   KLU refactor          src/klu_native/refactor.rs:68-152, kernel.rs:476-524
 *   KLU solve             src/klu_native/solve.rs:56-102
 *   newton_raphson_cached src/solver.rs:639-736
 *   BatchSolver::solve    src/batch.rs:198-289 (work queue, one solver per worker)
 *
 * The symbolic ordering (BTF + AMD: P, Q, R) is an INPUT here.  It is pinned
 * separately against the reference's compiled klu_analyze.
 */
#ifndef GOX_ORACLE_H
#define GOX_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define GXO_PQ 1
#define GXO_PV 2
#define GXO_SLACK 3

#define GXO_CONVERGED 0
#define GXO_MAXITER 1
#define GXO_SINGULAR 2

/* Y-bus: returns nnz; rowptr [n+1], col/yre/yim capacity n + 4m. */
int gxo_ybus_build(int n, int m, const int32_t *from, const int32_t *to, const double *r,
                   const double *x, const double *b, const double *tap,
                   const uint8_t *is_trafo, int32_t *rowptr, int32_t *col, double *yre,
                   double *yim);

void gxo_injections(int n, const int32_t *yp, const int32_t *yi, const double *yre,
                    const double *yim, const double *vm, const double *va, double *p,
                    double *q);

/* Jacobian pattern in the reference's emission order. */
typedef struct gxo_jac gxo_jac;
gxo_jac *gxo_jac_analyze(int n, const int32_t *yp, const int32_t *yi, const int32_t *bus_type);
void gxo_jac_free(gxo_jac *j);
int gxo_jac_nnz(const gxo_jac *j);
int gxo_jac_nu(const gxo_jac *j);
/* rows, cols, kind, bus i, bus k, Y slot -- each [nnz] (NULL to skip) */
void gxo_jac_pattern(const gxo_jac *j, int32_t *rows, int32_t *cols, int32_t *kind,
                     int32_t *bi, int32_t *bk, int32_t *yslot);
void gxo_jac_fill(const gxo_jac *j, const double *yre, const double *yim, const double *vm,
                  const double *va, const double *p, const double *q, double *values);

/* KLU numeric restatement on a fixed symbolic ordering. */
typedef struct gxo_lu gxo_lu;
/* triplets (rows, cols) in a fixed order; values positionally matching.
 * P, Q: [n]; R: [nblocks+1].  Factors once with partial pivoting (tol 0.001,
 * diagonal preference).  Returns NULL on singular/invalid (*status set). */
gxo_lu *gxo_lu_new(int n, int nnz, const int32_t *rows, const int32_t *cols,
                   const double *vals, const int32_t *P, const int32_t *Q, const int32_t *R,
                   int nblocks, int *status);
void gxo_lu_free(gxo_lu *lu);
/* refactor (static pivots) + solve.  0 = ok, 1 = singular/non-finite. */
int gxo_lu_factor_solve_values(gxo_lu *lu, const double *vals, const double *rhs, double *x);
int gxo_lu_refactor(gxo_lu *lu, const double *vals);
int gxo_lu_solve(gxo_lu *lu, const double *rhs, double *x);
/* out: [0]=lnz incl diag, [1]=unz incl diag, [2]=nzoff, [3]=nblocks */
void gxo_lu_sizes(const gxo_lu *lu, int32_t *out);
/* Factors in klu_extract's layout: L unit-diag first per column, U diag last
 * per column, rows in final pivot order; Pnum, Q, R. */
void gxo_lu_extract(const gxo_lu *lu, int32_t *Lp, int32_t *Li, double *Lx, int32_t *Up,
                    int32_t *Ui, double *Ux, int32_t *Fp, int32_t *Fi, double *Fx,
                    int32_t *Pnum, int32_t *Q, int32_t *R);

/* One topology: Y-bus + bus types + Jacobian ordering. */
typedef struct gxo_topo gxo_topo;
gxo_topo *gxo_topo_new(int n, const int32_t *yp, const int32_t *yi, const double *yre,
                       const double *yim, const int32_t *bus_type, const int32_t *P,
                       const int32_t *Q, const int32_t *R, int nblocks);
void gxo_topo_free(gxo_topo *t);
/* ZIP terms of effective_injection (src/network.rs:600-611), [n] each; NULL clears. */
void gxo_topo_set_zip(gxo_topo *t, const double *zi_re, const double *zi_im, const double *zc_re,
                      const double *zc_im);

/* newton_raphson_cached for one scenario.  *cache holds the worker's
 * persistent LU (created on the first Jacobian it sees).  yre/yim: this
 * scenario's Y values (NULL = topology's).  vm, va in/out.  hist [max_iter]
 * or NULL.  Returns GXO_* status; *iters = len(history). */
int gxo_nr_solve(gxo_topo *t, gxo_lu **cache, const double *yre, const double *yim,
                 double *vm, double *va, const double *p_spec, const double *q_spec,
                 double tol, int max_iter, double *hist, int *iters);

/* BatchSolver::solve: B scenarios, nthreads workers each with its own
 * persistent LU.  p_spec/q_spec [B][N]; vm0/va0 start voltages with row
 * stride v_stride (0 = shared template).  Optional outage deltas: dslot
 * [B][4] Y slots, dre/dim [B][4] values added to them (NULL = none).
 * Outputs [B][N] voltages and per-scenario iters/status/final mismatch;
 * hist [B][max_iter] or NULL. */
int gxo_batch_solve(gxo_topo *t, int B, const double *p_spec, const double *q_spec,
                    const double *vm0, const double *va0, int v_stride, const int32_t *dslot,
                    const double *dre, const double *dim, double tol, int max_iter,
                    int nthreads, double *vm_out, double *va_out, int32_t *iters,
                    int32_t *status, double *max_mis, double *hist);

#ifdef __cplusplus
}
#endif
#endif
