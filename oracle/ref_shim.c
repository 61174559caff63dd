/*
 * ref_shim.c -- TEST INFRASTRUCTURE ONLY (oracle side; never linked into the
 * product library).
 *
 * A flat C wrapper around the reference's vendored SuiteSparse KLU
 * (gridoxide vendor/suitesparse, v7.12.2), compiled together with those
 * sources into oracle/_ref/libklu_ref.so by oracle/Makefile.  It exposes the
 * handful of calls the oracle tests need through plain pointers so ctypes can
 * drive them without mirroring klu_common:
 *
 *   - the symbolic ordering (klu_analyze: BTF + per-block AMD), i.e.
 *     Symbolic->P, Q, R -- what KluNative's analyze::analyze reproduces
 *     (gridoxide src/klu_native/analyze.rs:67-150);
 *   - the first numeric factorization with partial pivoting (klu_factor,
 *     tol 0.001) and its extracted factors (klu_extract), i.e. what
 *     KluNative's factor::factor produces (src/klu_native/factor.rs:47-131);
 *   - refactor + solve (klu_refactor, klu_solve), i.e. KluNative's
 *     factor_and_solve_values (src/klu_native/mod.rs:185-210).
 *
 * Common.scale is set to 0 (no row scaling) because KluNative runs unscaled
 * (src/klu_native/mod.rs:44-58; klu_factor.c applies Rs only when scale > 0).
 */
#include <stdlib.h>
#include <string.h>
#include "klu.h"

typedef struct {
    klu_common common;
    klu_symbolic *sym;
    klu_numeric *num;
    int n;
    int32_t *Ap, *Ai;
} ref_klu;

static void ref_defaults(klu_common *c) {
    klu_defaults(c);
    c->scale = 0;
}

/* Symbolic analysis only.  P, Q: size n; R: size n+1. Returns nblocks, or <0. */
int ref_analyze(int n, const int32_t *Ap, const int32_t *Ai,
                int32_t *P, int32_t *Q, int32_t *R) {
    klu_common c;
    ref_defaults(&c);
    klu_symbolic *s = klu_analyze(n, (int32_t *)Ap, (int32_t *)Ai, &c);
    if (!s) return -100 + c.status;
    memcpy(P, s->P, sizeof(int32_t) * n);
    memcpy(Q, s->Q, sizeof(int32_t) * n);
    int nb = s->nblocks;
    memcpy(R, s->R, sizeof(int32_t) * (nb + 1));
    klu_free_symbolic(&s, &c);
    return nb;
}

/* analyze + factor; returns handle or NULL (status in *status). */
void *ref_new(int n, const int32_t *Ap, const int32_t *Ai, const double *Ax, int *status) {
    ref_klu *h = (ref_klu *)calloc(1, sizeof(ref_klu));
    ref_defaults(&h->common);
    h->n = n;
    int nnz = Ap[n];
    h->Ap = (int32_t *)malloc(sizeof(int32_t) * (n + 1));
    h->Ai = (int32_t *)malloc(sizeof(int32_t) * (nnz > 0 ? nnz : 1));
    memcpy(h->Ap, Ap, sizeof(int32_t) * (n + 1));
    memcpy(h->Ai, Ai, sizeof(int32_t) * nnz);
    h->sym = klu_analyze(n, h->Ap, h->Ai, &h->common);
    if (!h->sym) { *status = h->common.status; free(h->Ap); free(h->Ai); free(h); return NULL; }
    h->num = klu_factor(h->Ap, h->Ai, (double *)Ax, h->sym, &h->common);
    if (!h->num) {
        *status = h->common.status;
        klu_free_symbolic(&h->sym, &h->common);
        free(h->Ap); free(h->Ai); free(h);
        return NULL;
    }
    *status = h->common.status;
    return h;
}

void ref_free(void *hv) {
    ref_klu *h = (ref_klu *)hv;
    if (!h) return;
    klu_free_numeric(&h->num, &h->common);
    klu_free_symbolic(&h->sym, &h->common);
    free(h->Ap); free(h->Ai); free(h);
}

/* Sizes of the extracted factors: out[0]=lnz (incl. unit diag), out[1]=unz
 * (incl. diag), out[2]=nzoff, out[3]=nblocks. */
void ref_sizes(void *hv, int32_t *out) {
    ref_klu *h = (ref_klu *)hv;
    out[0] = h->num->lnz; out[1] = h->num->unz; out[2] = h->num->nzoff; out[3] = h->sym->nblocks;
}

/* Symbolic P,Q,R of the handle. */
void ref_symbolic(void *hv, int32_t *P, int32_t *Q, int32_t *R) {
    ref_klu *h = (ref_klu *)hv;
    memcpy(P, h->sym->P, sizeof(int32_t) * h->n);
    memcpy(Q, h->sym->Q, sizeof(int32_t) * h->n);
    memcpy(R, h->sym->R, sizeof(int32_t) * (h->sym->nblocks + 1));
}

int ref_extract(void *hv, int32_t *Lp, int32_t *Li, double *Lx, int32_t *Up, int32_t *Ui, double *Ux,
                int32_t *Fp, int32_t *Fi, double *Fx, int32_t *P, int32_t *Q, int32_t *R) {
    ref_klu *h = (ref_klu *)hv;
    return klu_extract(h->num, h->sym, Lp, Li, Lx, Up, Ui, Ux, Fp, Fi, Fx, P, Q, NULL, R, &h->common);
}

/* klu_refactor on new values (same pattern), then klu_solve in place on b.
 * Returns common.status (0 ok, 1 singular) or <0 on error. */
int ref_refactor_solve(void *hv, const double *Ax, double *b) {
    ref_klu *h = (ref_klu *)hv;
    if (!klu_refactor(h->Ap, h->Ai, (double *)Ax, h->sym, h->num, &h->common)) return h->common.status ? h->common.status : -1;
    if (!klu_solve(h->sym, h->num, h->n, 1, b, &h->common)) return h->common.status ? h->common.status : -1;
    return h->common.status;
}

int ref_refactor(void *hv, const double *Ax) {
    ref_klu *h = (ref_klu *)hv;
    if (!klu_refactor(h->Ap, h->Ai, (double *)Ax, h->sym, h->num, &h->common)) return h->common.status ? h->common.status : -1;
    return h->common.status;
}

int ref_solve(void *hv, double *b) {
    ref_klu *h = (ref_klu *)hv;
    if (!klu_solve(h->sym, h->num, h->n, 1, b, &h->common)) return h->common.status ? h->common.status : -1;
    return h->common.status;
}
