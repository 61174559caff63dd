/*
 * gox_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * Plain-C CPU restatement of the reference's batched Newton-Raphson path;
 * see gox_oracle.h for the file:line each part follows.  It is the checker
 * for the GPU engine (tests, smoke) and the timed CPU baseline (bench.py);
 * the product library never links it.
 *
 * Build: make -C oracle (gcc -O2 -ffp-contract=off, identical results on
 * x86_64 and aarch64).
 */
#include "gox_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define EMPTY (-1)
#define FLIP(i) (-(i)-2)
#define UNFLIP(i) (((i) < EMPTY) ? FLIP(i) : (i))

static void *xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p) abort();
    return p;
}
static void *xcalloc(size_t n, size_t s) {
    void *p = calloc(n ? n : 1, s ? s : 1);
    if (!p) abort();
    return p;
}

/* num-complex 0.4 division: (a.re*b.re + a.im*b.im, a.im*b.re - a.re*b.im)/|b|^2 */
static void cdiv(double ar, double ai, double br, double bi, double *cr, double *ci) {
    double n = br * br + bi * bi;
    *cr = (ar * br + ai * bi) / n;
    *ci = (ai * br - ar * bi) / n;
}

/* ------------------------------------------------------------------------ */
/* Y-bus (src/network.rs:225-247 lines, 339-373 transformers, 52-71 finish)  */

typedef struct {
    int32_t r, c, ord;
    double re, im;
} trip_t;

static int trip_cmp(const void *a, const void *b) {
    const trip_t *x = (const trip_t *)a, *y = (const trip_t *)b;
    if (x->r != y->r) return x->r < y->r ? -1 : 1;
    if (x->c != y->c) return x->c < y->c ? -1 : 1;
    return x->ord < y->ord ? -1 : (x->ord > y->ord);
}

int gxo_ybus_build(int n, int m, const int32_t *from, const int32_t *to, const double *r,
                   const double *x, const double *b, const double *tap,
                   const uint8_t *is_trafo, int32_t *rowptr, int32_t *col, double *yre,
                   double *yim) {
    trip_t *t = (trip_t *)xmalloc(sizeof(trip_t) * (size_t)(4 * m + 1));
    int nt = 0;
#define ADD(R_, C_, RE_, IM_)                                                            \
    do {                                                                                 \
        t[nt].r = (R_); t[nt].c = (C_); t[nt].re = (RE_); t[nt].im = (IM_);             \
        t[nt].ord = nt; nt++;                                                           \
    } while (0)
    /* lines first (build_ybus), then transformers (stamp_transformers) */
    for (int pass = 0; pass < 2; pass++) {
        for (int e = 0; e < m; e++) {
            int tr = is_trafo ? is_trafo[e] != 0 : 0;
            if (tr != pass) continue;
            int f = from[e], o = to[e];
            if (!tr) {
                if (f == o) { /* pure shunt */
                    ADD(f, f, 0.0, b[e]);
                    continue;
                }
                double yr, yi;
                cdiv(1.0, 0.0, r[e], x[e], &yr, &yi);
                double hr = 0.0 / 2.0, hi = b[e] / 2.0;
                ADD(f, f, yr + hr, yi + hi);
                ADD(o, o, yr + hr, yi + hi);
                ADD(f, o, -yr, -yi);
                ADD(o, f, -yr, -yi);
            } else {
                double ysr, ysi;
                cdiv(1.0, 0.0, r[e], x[e], &ysr, &ysi);
                double shr = 0.0, shi = b[e];
                double k = fabs(tap[e]);
                double ydr = ysr + shr * 0.5, ydi = ysi + shi * 0.5;
                double ffr = ydr / (k * k), ffi = ydi / (k * k);
                double ftr, fti, tfr, tfi;
                cdiv(-ysr, -ysi, tap[e], -0.0, &ftr, &fti); /* -y_s / conj(t) */
                cdiv(-ysr, -ysi, tap[e], 0.0, &tfr, &tfi);  /* -y_s / t */
                ADD(f, f, ffr, ffi);
                ADD(f, o, ftr, fti);
                ADD(o, f, tfr, tfi);
                ADD(o, o, ydr, ydi);
            }
        }
    }
#undef ADD
    qsort(t, (size_t)nt, sizeof(trip_t), trip_cmp);
    int nnz = 0;
    for (int i = 0; i <= n; i++) rowptr[i] = 0;
    for (int p = 0; p < nt;) {
        int q = p;
        double sr = 0.0, si = 0.0;
        while (q < nt && t[q].r == t[p].r && t[q].c == t[p].c) {
            sr += t[q].re;
            si += t[q].im;
            q++;
        }
        col[nnz] = t[p].c;
        yre[nnz] = sr;
        yim[nnz] = si;
        rowptr[t[p].r + 1]++;
        nnz++;
        p = q;
    }
    for (int i = 0; i < n; i++) rowptr[i + 1] += rowptr[i];
    free(t);
    return nnz;
}

/* ------------------------------------------------------------------------ */
/* power_injections (src/network.rs:680-701)                                 */

void gxo_injections(int n, const int32_t *yp, const int32_t *yi, const double *yre,
                    const double *yim, const double *vm, const double *va, double *p,
                    double *q) {
    for (int i = 0; i < n; i++) {
        double ir = 0.0, ii = 0.0;
        for (int s = yp[i]; s < yp[i + 1]; s++) {
            int k = yi[s];
            double vr = vm[k] * cos(va[k]), vi = vm[k] * sin(va[k]);
            ir += yre[s] * vr - yim[s] * vi;
            ii += yre[s] * vi + yim[s] * vr;
        }
        double vr = vm[i] * cos(va[i]), vi = vm[i] * sin(va[i]);
        /* S = v * conj(I) */
        p[i] = vr * ir - vi * (-ii);
        q[i] = vr * (-ii) + vi * ir;
    }
}

/* ------------------------------------------------------------------------ */
/* JacobianPattern (src/jacobian.rs:48-57 kinds, 96-171 analyze, 202-250 fill) */

enum { K_HII = 0, K_NII = 1, K_HIK = 2, K_NIK = 3, K_MII = 4, K_LII = 5, K_MIK = 6, K_LIK = 7 };

struct gxo_jac {
    int n_bus, n_ang, n_u, nnz;
    int32_t *rows, *cols, *kind, *bi, *bk, *yslot;
};

gxo_jac *gxo_jac_analyze(int n, const int32_t *yp, const int32_t *yi, const int32_t *bus_type) {
    gxo_jac *j = (gxo_jac *)xcalloc(1, sizeof(gxo_jac));
    int32_t *ns_pos = (int32_t *)xmalloc(sizeof(int32_t) * n);
    int32_t *pq_pos = (int32_t *)xmalloc(sizeof(int32_t) * n);
    int n_ang = 0, n_pq = 0;
    for (int i = 0; i < n; i++) ns_pos[i] = bus_type[i] != GXO_SLACK ? n_ang++ : -1;
    for (int i = 0; i < n; i++) pq_pos[i] = bus_type[i] == GXO_PQ ? n_pq++ : -1;
    int cap = 2 * yp[n] * 2 + 4;
    j->rows = (int32_t *)xmalloc(sizeof(int32_t) * cap);
    j->cols = (int32_t *)xmalloc(sizeof(int32_t) * cap);
    j->kind = (int32_t *)xmalloc(sizeof(int32_t) * cap);
    j->bi = (int32_t *)xmalloc(sizeof(int32_t) * cap);
    j->bk = (int32_t *)xmalloc(sizeof(int32_t) * cap);
    j->yslot = (int32_t *)xmalloc(sizeof(int32_t) * cap);
    int e = 0;
#define PUSH(R_, C_, K_, I_, KK_, S_)                                                    \
    do {                                                                                 \
        j->rows[e] = (R_); j->cols[e] = (C_); j->kind[e] = (K_);                        \
        j->bi[e] = (I_); j->bk[e] = (KK_); j->yslot[e] = (S_); e++;                     \
    } while (0)
    /* H and N rows: non-slack buses in bus order */
    for (int i = 0; i < n; i++) {
        if (ns_pos[i] < 0) continue;
        int row = ns_pos[i];
        for (int s = yp[i]; s < yp[i + 1]; s++) {
            int k = yi[s];
            if (k == i) {
                PUSH(row, row, K_HII, i, i, s);
                if (pq_pos[i] >= 0) PUSH(row, n_ang + pq_pos[i], K_NII, i, i, s);
                continue;
            }
            if (ns_pos[k] >= 0) PUSH(row, ns_pos[k], K_HIK, i, k, s);
            if (pq_pos[k] >= 0) PUSH(row, n_ang + pq_pos[k], K_NIK, i, k, s);
        }
    }
    /* M and L rows: PQ buses in bus order */
    for (int i = 0; i < n; i++) {
        if (pq_pos[i] < 0) continue;
        int row = n_ang + pq_pos[i];
        for (int s = yp[i]; s < yp[i + 1]; s++) {
            int k = yi[s];
            if (k == i) {
                PUSH(row, ns_pos[i], K_MII, i, i, s);
                PUSH(row, row, K_LII, i, i, s);
                continue;
            }
            if (ns_pos[k] >= 0) PUSH(row, ns_pos[k], K_MIK, i, k, s);
            if (pq_pos[k] >= 0) PUSH(row, n_ang + pq_pos[k], K_LIK, i, k, s);
        }
    }
#undef PUSH
    j->n_bus = n;
    j->n_ang = n_ang;
    j->n_u = n_ang + n_pq;
    j->nnz = e;
    free(ns_pos);
    free(pq_pos);
    return j;
}

void gxo_jac_free(gxo_jac *j) {
    if (!j) return;
    free(j->rows); free(j->cols); free(j->kind); free(j->bi); free(j->bk); free(j->yslot);
    free(j);
}
int gxo_jac_nnz(const gxo_jac *j) { return j->nnz; }
int gxo_jac_nu(const gxo_jac *j) { return j->n_u; }

void gxo_jac_pattern(const gxo_jac *j, int32_t *rows, int32_t *cols, int32_t *kind,
                     int32_t *bi, int32_t *bk, int32_t *yslot) {
    size_t sz = sizeof(int32_t) * (size_t)j->nnz;
    if (rows) memcpy(rows, j->rows, sz);
    if (cols) memcpy(cols, j->cols, sz);
    if (kind) memcpy(kind, j->kind, sz);
    if (bi) memcpy(bi, j->bi, sz);
    if (bk) memcpy(bk, j->bk, sz);
    if (yslot) memcpy(yslot, j->yslot, sz);
}

void gxo_jac_fill(const gxo_jac *j, const double *yre, const double *yim, const double *vm,
                  const double *va, const double *p, const double *q, double *values) {
    for (int e = 0; e < j->nnz; e++) {
        int i = j->bi[e], k = j->bk[e], s = j->yslot[e];
        double vm_i = vm[i], g = yre[s], b = yim[s], v;
        switch (j->kind[e]) {
        case K_HII: v = -q[i] - (vm_i * vm_i) * b; break;
        case K_NII: v = p[i] / vm_i + vm_i * g; break;
        case K_MII: v = p[i] - (vm_i * vm_i) * g; break;
        case K_LII: v = q[i] / vm_i - vm_i * b; break;
        default: {
            double vm_k = vm[k];
            double ang = va[i] - va[k];
            double sn = sin(ang), cs = cos(ang);
            switch (j->kind[e]) {
            case K_HIK: v = vm_i * vm_k * (g * sn - b * cs); break;
            case K_NIK: v = vm_i * (g * cs + b * sn); break;
            case K_MIK: v = -vm_i * vm_k * (g * cs + b * sn); break;
            default: v = vm_i * (g * sn - b * cs); break; /* K_LIK */
            }
        }
        }
        values[e] = v;
    }
}

/* ------------------------------------------------------------------------ */
/* KLU numeric restatement                                                   */

struct gxo_lu {
    int n, nnz, nblocks;
    int32_t *Ap, *Ai;          /* CSC pattern of the triplets (build_csc_structure) */
    int32_t *gp, *gi;          /* groups: triplet indices per CSC slot */
    double *Ax;                /* packed CSC values */
    int32_t *P, *Q, *R;        /* symbolic ordering */
    int32_t *Pnum, *Pinv;      /* final numeric row permutation */
    int32_t *Lip, *Llen, *Uip, *Ulen; /* per global column, into Li/Ui (block-local rows) */
    int32_t *Li, *Ui;
    double *Lx, *Ux, *Udiag;
    int lcap, ucap, lnext, unext;
    int32_t *Offp, *Offi;
    double *Offx;
    int nzoff, offcap;
    double *X;
};

typedef struct {
    int32_t r, c, ord;
} pair_t;
static int pair_cmp_colrow(const void *a, const void *b) {
    const pair_t *x = (const pair_t *)a, *y = (const pair_t *)b;
    if (x->c != y->c) return x->c < y->c ? -1 : 1;
    if (x->r != y->r) return x->r < y->r ? -1 : 1;
    return x->ord < y->ord ? -1 : (x->ord > y->ord);
}

/* build_csc_structure (src/klu_native/mod.rs:88-114) */
static void build_csc(gxo_lu *lu, int nnzt, const int32_t *rows, const int32_t *cols) {
    int n = lu->n;
    pair_t *pp = (pair_t *)xmalloc(sizeof(pair_t) * (size_t)(nnzt + 1));
    for (int e = 0; e < nnzt; e++) { pp[e].r = rows[e]; pp[e].c = cols[e]; pp[e].ord = e; }
    qsort(pp, (size_t)nnzt, sizeof(pair_t), pair_cmp_colrow);
    lu->Ap = (int32_t *)xcalloc((size_t)n + 1, sizeof(int32_t));
    lu->Ai = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nnzt + 1));
    lu->gp = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nnzt + 2));
    lu->gi = (int32_t *)xmalloc(sizeof(int32_t) * (size_t)(nnzt + 1));
    int ns = 0;
    lu->gp[0] = 0;
    for (int p = 0; p < nnzt;) {
        int q = p;
        while (q < nnzt && pp[q].r == pp[p].r && pp[q].c == pp[p].c) {
            lu->gi[q] = pp[q].ord;
            q++;
        }
        lu->Ai[ns] = pp[p].r;
        lu->Ap[pp[p].c + 1]++;
        ns++;
        lu->gp[ns] = q;
        p = q;
    }
    for (int c = 0; c < n; c++) lu->Ap[c + 1] += lu->Ap[c];
    lu->nnz = ns;
    lu->Ax = (double *)xmalloc(sizeof(double) * (size_t)(ns + 1));
    free(pp);
}

static void pack_values(gxo_lu *lu, const double *vals) {
    for (int s = 0; s < lu->nnz; s++) {
        double acc = 0.0;
        for (int p = lu->gp[s]; p < lu->gp[s + 1]; p++) acc += vals[lu->gi[p]];
        lu->Ax[s] = acc;
    }
}

static void grow_l(gxo_lu *lu, int need) {
    if (lu->lnext + need <= lu->lcap) return;
    int nc = (lu->lcap * 2 > lu->lnext + need) ? lu->lcap * 2 : lu->lnext + need + 16;
    lu->Li = (int32_t *)realloc(lu->Li, sizeof(int32_t) * nc);
    lu->Lx = (double *)realloc(lu->Lx, sizeof(double) * nc);
    if (!lu->Li || !lu->Lx) abort();
    lu->lcap = nc;
}
static void grow_u(gxo_lu *lu, int need) {
    if (lu->unext + need <= lu->ucap) return;
    int nc = (lu->ucap * 2 > lu->unext + need) ? lu->ucap * 2 : lu->unext + need + 16;
    lu->Ui = (int32_t *)realloc(lu->Ui, sizeof(int32_t) * nc);
    lu->Ux = (double *)realloc(lu->Ux, sizeof(double) * nc);
    if (!lu->Ui || !lu->Ux) abort();
    lu->ucap = nc;
}

/* Non-recursive DFS (klu_kernel.c dfs; src/klu_native/kernel.rs:32-93).
 * Column j's L rows live at Li[Lip[k1+jnew] ...]. */
static int kdfs(gxo_lu *lu, int k1, int j, int k, const int32_t *Pinv, int32_t *Stack,
                int32_t *Flag, const int32_t *Lpend, int top, int32_t *Lik, int *plen,
                int32_t *Ap_pos) {
    int head = 0, l_length = *plen;
    Stack[0] = j;
    while (head >= 0) {
        j = Stack[head];
        int jnew = Pinv[j];
        if (Flag[j] != k) {
            Flag[j] = k;
            Ap_pos[head] = (Lpend[jnew] == EMPTY) ? lu->Llen[k1 + jnew] : Lpend[jnew];
        }
        const int32_t *Lj = lu->Li + lu->Lip[k1 + jnew];
        int pos;
        for (pos = --Ap_pos[head]; pos >= 0; --pos) {
            int i = Lj[pos];
            if (Flag[i] != k) {
                if (Pinv[i] >= 0) {
                    Ap_pos[head] = pos;
                    Stack[++head] = i;
                    break;
                } else {
                    Flag[i] = k;
                    Lik[l_length++] = i;
                }
            }
        }
        if (pos == -1) {
            head--;
            Stack[--top] = j;
        }
    }
    *plen = l_length;
    return top;
}

/* KLU_kernel for one block [k1, k2) (klu_kernel.c; kernel.rs:341-416).
 * Returns 1 on success, 0 if singular.  Pblk [nk] = block-local pivot rows. */
static int factor_block(gxo_lu *lu, int k1, int k2, const int32_t *PSinv, int32_t *Pblk,
                        double tol) {
    int nk = k2 - k1;
    int32_t *Pinv = (int32_t *)xmalloc(sizeof(int32_t) * nk);
    int32_t *Flag = (int32_t *)xmalloc(sizeof(int32_t) * nk);
    int32_t *Lpend = (int32_t *)xmalloc(sizeof(int32_t) * nk);
    int32_t *Stack = (int32_t *)xmalloc(sizeof(int32_t) * nk);
    int32_t *Ap_pos = (int32_t *)xmalloc(sizeof(int32_t) * nk);
    double *X = (double *)xcalloc((size_t)nk, sizeof(double));
    int ok = 1;
    for (int k = 0; k < nk; k++) {
        Flag[k] = EMPTY;
        Lpend[k] = EMPTY;
        Pblk[k] = k;
        Pinv[k] = FLIP(k);
    }
    for (int k = 0; k < nk; k++) {
        int kg = k + k1;
        grow_l(lu, nk);
        lu->Lip[kg] = lu->lnext;
        int32_t *Lik = lu->Li + lu->lnext;
        /* lsolve_symbolic */
        int top = nk, l_length = 0;
        int oldcol = lu->Q[kg];
        for (int p = lu->Ap[oldcol]; p < lu->Ap[oldcol + 1]; p++) {
            int i = PSinv[lu->Ai[p]] - k1;
            if (i < 0) continue;
            if (Flag[i] != k) {
                if (Pinv[i] >= 0) {
                    top = kdfs(lu, k1, i, k, Pinv, Stack, Flag, Lpend, top, Lik, &l_length,
                               Ap_pos);
                } else {
                    Flag[i] = k;
                    Lik[l_length++] = i;
                }
            }
        }
        lu->Llen[kg] = l_length;
        /* construct_column (unscaled) */
        int poff = lu->Offp[kg];
        for (int p = lu->Ap[oldcol]; p < lu->Ap[oldcol + 1]; p++) {
            int oldrow = lu->Ai[p];
            int i = PSinv[oldrow] - k1;
            if (i < 0) {
                if (poff >= lu->offcap) {
                    lu->offcap = lu->offcap * 2 + 16;
                    lu->Offi = (int32_t *)realloc(lu->Offi, sizeof(int32_t) * lu->offcap);
                    lu->Offx = (double *)realloc(lu->Offx, sizeof(double) * lu->offcap);
                }
                lu->Offi[poff] = oldrow;
                lu->Offx[poff] = lu->Ax[p];
                poff++;
            } else {
                X[i] = lu->Ax[p];
            }
        }
        lu->Offp[kg + 1] = poff;
        /* lsolve_numeric */
        for (int s = top; s < nk; s++) {
            int j = Stack[s];
            int jnew = Pinv[j];
            double xj = X[j];
            const int32_t *Lj = lu->Li + lu->Lip[k1 + jnew];
            const double *Lxj = lu->Lx + lu->Lip[k1 + jnew];
            int len = lu->Llen[k1 + jnew];
            for (int p = 0; p < len; p++) X[Lj[p]] -= Lxj[p] * xj;
        }
        /* lpivot */
        int diagrow = Pblk[k];
        int pivrow;
        double pivot;
        if (lu->Llen[kg] == 0) { ok = 0; break; }
        {
            int pdiag = EMPTY, ppivrow = EMPTY;
            double abs_pivot = EMPTY, xabs;
            int ii = lu->Llen[kg] - 1;
            int32_t *Li = lu->Li + lu->Lip[kg];
            double *Lx = lu->Lx + lu->Lip[kg];
            int last_row_index = Li[ii];
            lu->Llen[kg] = ii;
            int len = ii;
            for (int p = 0; p < len; p++) {
                int i = Li[p];
                double x = X[i];
                X[i] = 0.0;
                Lx[p] = x;
                xabs = fabs(x);
                if (i == diagrow) pdiag = p;
                if (xabs > abs_pivot) { abs_pivot = xabs; ppivrow = p; }
            }
            xabs = fabs(X[last_row_index]);
            if (xabs > abs_pivot) { abs_pivot = xabs; ppivrow = EMPTY; }
            if (last_row_index == diagrow) {
                if (xabs >= tol * abs_pivot) { abs_pivot = xabs; ppivrow = EMPTY; }
            } else if (pdiag != EMPTY) {
                xabs = fabs(Lx[pdiag]);
                if (xabs >= tol * abs_pivot) { abs_pivot = xabs; ppivrow = pdiag; }
            }
            if (ppivrow != EMPTY) {
                pivrow = Li[ppivrow];
                pivot = Lx[ppivrow];
                Li[ppivrow] = last_row_index;
                Lx[ppivrow] = X[last_row_index];
            } else {
                pivrow = last_row_index;
                pivot = X[last_row_index];
            }
            X[last_row_index] = 0.0;
            if (pivot == 0.0) { ok = 0; break; }
            for (int p = 0; p < lu->Llen[kg]; p++) Lx[p] /= pivot;
        }
        lu->lnext += lu->Llen[kg];
        /* U(:,k) = X[Stack[top..nk)] */
        grow_u(lu, nk - top);
        lu->Uip[kg] = lu->unext;
        lu->Ulen[kg] = nk - top;
        {
            int32_t *Ui = lu->Ui + lu->Uip[kg];
            double *Ux = lu->Ux + lu->Uip[kg];
            for (int p = top, i = 0; p < nk; p++, i++) {
                int j = Stack[p];
                Ui[i] = Pinv[j];
                Ux[i] = X[j];
                X[j] = 0.0;
            }
        }
        lu->unext += nk - top;
        lu->Udiag[kg] = pivot;
        if (pivrow != diagrow) {
            if (Pinv[diagrow] < 0) {
                int kbar = FLIP(Pinv[pivrow]);
                Pblk[kbar] = diagrow;
                Pinv[diagrow] = FLIP(kbar);
            }
        }
        Pblk[k] = pivrow;
        Pinv[pivrow] = k;
        /* prune (klu_kernel.c prune; kernel.rs:270-291) */
        {
            const int32_t *Ui = lu->Ui + lu->Uip[kg];
            for (int p = 0; p < lu->Ulen[kg]; p++) {
                int j = Ui[p];
                if (Lpend[j] != EMPTY) continue;
                int32_t *Li = lu->Li + lu->Lip[k1 + j];
                double *Lx = lu->Lx + lu->Lip[k1 + j];
                int llen = lu->Llen[k1 + j];
                for (int p2 = 0; p2 < llen; p2++) {
                    if (pivrow == Li[p2]) {
                        int phead = 0, ptail = llen;
                        while (phead < ptail) {
                            int i = Li[phead];
                            if (Pinv[i] >= 0) {
                                phead++;
                            } else {
                                ptail--;
                                Li[phead] = Li[ptail];
                                Li[ptail] = i;
                                double x = Lx[phead];
                                Lx[phead] = Lx[ptail];
                                Lx[ptail] = x;
                            }
                        }
                        Lpend[j] = ptail;
                        break;
                    }
                }
            }
        }
    }
    if (ok) {
        /* renumber L rows to pivot positions */
        for (int k = 0; k < nk; k++) {
            int32_t *Li = lu->Li + lu->Lip[k1 + k];
            for (int p = 0; p < lu->Llen[k1 + k]; p++) Li[p] = Pinv[Li[p]];
        }
    }
    free(Pinv); free(Flag); free(Lpend); free(Stack); free(Ap_pos); free(X);
    return ok;
}

gxo_lu *gxo_lu_new(int n, int nnz, const int32_t *rows, const int32_t *cols,
                   const double *vals, const int32_t *P, const int32_t *Q, const int32_t *R,
                   int nblocks, int *status) {
    gxo_lu *lu = (gxo_lu *)xcalloc(1, sizeof(gxo_lu));
    lu->n = n;
    lu->nblocks = nblocks;
    build_csc(lu, nnz, rows, cols);
    pack_values(lu, vals);
    lu->P = (int32_t *)xmalloc(sizeof(int32_t) * n);
    lu->Q = (int32_t *)xmalloc(sizeof(int32_t) * n);
    lu->R = (int32_t *)xmalloc(sizeof(int32_t) * (nblocks + 1));
    memcpy(lu->P, P, sizeof(int32_t) * n);
    memcpy(lu->Q, Q, sizeof(int32_t) * n);
    memcpy(lu->R, R, sizeof(int32_t) * (nblocks + 1));
    lu->Pnum = (int32_t *)xmalloc(sizeof(int32_t) * n);
    lu->Pinv = (int32_t *)xmalloc(sizeof(int32_t) * n);
    lu->Lip = (int32_t *)xcalloc(n, sizeof(int32_t));
    lu->Llen = (int32_t *)xcalloc(n, sizeof(int32_t));
    lu->Uip = (int32_t *)xcalloc(n, sizeof(int32_t));
    lu->Ulen = (int32_t *)xcalloc(n, sizeof(int32_t));
    lu->Udiag = (double *)xcalloc(n, sizeof(double));
    lu->lcap = lu->ucap = 4 * lu->nnz + 16;
    lu->Li = (int32_t *)xmalloc(sizeof(int32_t) * lu->lcap);
    lu->Lx = (double *)xmalloc(sizeof(double) * lu->lcap);
    lu->Ui = (int32_t *)xmalloc(sizeof(int32_t) * lu->ucap);
    lu->Ux = (double *)xmalloc(sizeof(double) * lu->ucap);
    lu->Offp = (int32_t *)xcalloc((size_t)n + 1, sizeof(int32_t));
    lu->offcap = 16;
    lu->Offi = (int32_t *)xmalloc(sizeof(int32_t) * lu->offcap);
    lu->Offx = (double *)xmalloc(sizeof(double) * lu->offcap);
    lu->X = (double *)xcalloc((size_t)n + 1, sizeof(double));
    int32_t *PSinv = (int32_t *)xmalloc(sizeof(int32_t) * n);
    for (int k = 0; k < n; k++) PSinv[P[k]] = k;
    int32_t *Pblk = (int32_t *)xmalloc(sizeof(int32_t) * n);
    int ok = 1;
    for (int b = 0; b < nblocks && ok; b++) {
        int k1 = R[b], k2 = R[b + 1];
        ok = factor_block(lu, k1, k2, PSinv, Pblk, 0.001);
        if (!ok) break;
        for (int k = 0; k < k2 - k1; k++) lu->Pnum[k + k1] = P[Pblk[k] + k1];
    }
    free(PSinv);
    free(Pblk);
    if (!ok) {
        *status = 1;
        gxo_lu_free(lu);
        return NULL;
    }
    for (int k = 0; k < n; k++) lu->Pinv[lu->Pnum[k]] = k;
    lu->nzoff = lu->Offp[n];
    for (int p = 0; p < lu->nzoff; p++) lu->Offi[p] = lu->Pinv[lu->Offi[p]];
    *status = 0;
    return lu;
}

void gxo_lu_free(gxo_lu *lu) {
    if (!lu) return;
    free(lu->Ap); free(lu->Ai); free(lu->gp); free(lu->gi); free(lu->Ax);
    free(lu->P); free(lu->Q); free(lu->R); free(lu->Pnum); free(lu->Pinv);
    free(lu->Lip); free(lu->Llen); free(lu->Uip); free(lu->Ulen);
    free(lu->Li); free(lu->Ui); free(lu->Lx); free(lu->Ux); free(lu->Udiag);
    free(lu->Offp); free(lu->Offi); free(lu->Offx); free(lu->X);
    free(lu);
}

/* klu_refactor (unscaled; kernel.rs:476-524, refactor.rs:68-152) */
int gxo_lu_refactor(gxo_lu *lu, const double *vals) {
    pack_values(lu, vals);
    double *X = lu->X;
    int poff = 0;
    for (int b = 0; b < lu->nblocks; b++) {
        int k1 = lu->R[b], k2 = lu->R[b + 1], nk = k2 - k1;
        for (int k = 0; k < nk; k++) {
            int kg = k + k1;
            int oldcol = lu->Q[kg];
            for (int p = lu->Ap[oldcol]; p < lu->Ap[oldcol + 1]; p++) {
                int oldrow = lu->Ai[p];
                int newrow = lu->Pinv[oldrow] - k1;
                if (newrow < 0 && poff < lu->nzoff) {
                    lu->Offx[poff++] = lu->Ax[p];
                } else {
                    X[newrow] = lu->Ax[p];
                }
            }
            const int32_t *Ui = lu->Ui + lu->Uip[kg];
            double *Ux = lu->Ux + lu->Uip[kg];
            for (int up = 0; up < lu->Ulen[kg]; up++) {
                int j = Ui[up];
                double ujk = X[j];
                X[j] = 0.0;
                Ux[up] = ujk;
                const int32_t *Lj = lu->Li + lu->Lip[k1 + j];
                const double *Lxj = lu->Lx + lu->Lip[k1 + j];
                for (int p = 0; p < lu->Llen[k1 + j]; p++) X[Lj[p]] -= Lxj[p] * ujk;
            }
            double ukk = X[k];
            X[k] = 0.0;
            if (ukk == 0.0) {
                /* leave X clean for the next call */
                memset(X, 0, sizeof(double) * (size_t)lu->n);
                return 1;
            }
            lu->Udiag[kg] = ukk;
            const int32_t *Li = lu->Li + lu->Lip[kg];
            double *Lx = lu->Lx + lu->Lip[kg];
            for (int p = 0; p < lu->Llen[kg]; p++) {
                int i = Li[p];
                Lx[p] = X[i] / ukk;
                X[i] = 0.0;
            }
        }
    }
    return 0;
}

/* klu_solve (solve.rs:56-102): x = Q * (L U + Off) \ (P b) */
int gxo_lu_solve(gxo_lu *lu, const double *rhs, double *x) {
    int n = lu->n;
    double *X = (double *)xmalloc(sizeof(double) * (size_t)(n + 1));
    for (int k = 0; k < n; k++) X[k] = rhs[lu->Pnum[k]];
    for (int b = lu->nblocks - 1; b >= 0; b--) {
        int k1 = lu->R[b], k2 = lu->R[b + 1], nk = k2 - k1;
        double *Xb = X + k1;
        if (nk == 1) {
            Xb[0] /= lu->Udiag[k1];
        } else {
            for (int k = 0; k < nk; k++) { /* lsolve */
                double xk = Xb[k];
                const int32_t *Li = lu->Li + lu->Lip[k1 + k];
                const double *Lx = lu->Lx + lu->Lip[k1 + k];
                for (int p = 0; p < lu->Llen[k1 + k]; p++) Xb[Li[p]] -= Lx[p] * xk;
            }
            for (int k = nk - 1; k >= 0; k--) { /* usolve */
                double xk = Xb[k] / lu->Udiag[k1 + k];
                Xb[k] = xk;
                const int32_t *Ui = lu->Ui + lu->Uip[k1 + k];
                const double *Ux = lu->Ux + lu->Uip[k1 + k];
                for (int p = 0; p < lu->Ulen[k1 + k]; p++) Xb[Ui[p]] -= Ux[p] * xk;
            }
        }
        if (b > 0) {
            for (int k = k1; k < k2; k++) {
                double xk = X[k];
                for (int p = lu->Offp[k]; p < lu->Offp[k + 1]; p++)
                    X[lu->Offi[p]] -= lu->Offx[p] * xk;
            }
        }
    }
    int bad = 0;
    for (int k = 0; k < n; k++) {
        x[lu->Q[k]] = X[k];
        if (!isfinite(X[k])) bad = 1;
    }
    free(X);
    return bad;
}

int gxo_lu_factor_solve_values(gxo_lu *lu, const double *vals, const double *rhs, double *x) {
    if (gxo_lu_refactor(lu, vals)) return 1;
    return gxo_lu_solve(lu, rhs, x);
}

void gxo_lu_sizes(const gxo_lu *lu, int32_t *out) {
    int lnz = 0, unz = 0;
    for (int k = 0; k < lu->n; k++) {
        lnz += lu->Llen[k] + 1;
        unz += lu->Ulen[k] + 1;
    }
    out[0] = lnz; out[1] = unz; out[2] = lu->nzoff; out[3] = lu->nblocks;
}

void gxo_lu_extract(const gxo_lu *lu, int32_t *Lp, int32_t *Li, double *Lx, int32_t *Up,
                    int32_t *Ui, double *Ux, int32_t *Fp, int32_t *Fi, double *Fx,
                    int32_t *Pnum, int32_t *Q, int32_t *R) {
    int n = lu->n, nz = 0;
    for (int b = 0; b < lu->nblocks; b++) {
        int k1 = lu->R[b], k2 = lu->R[b + 1];
        for (int k = k1; k < k2; k++) {
            Lp[k] = nz;
            Li[nz] = k; Lx[nz] = 1.0; nz++;
            for (int p = 0; p < lu->Llen[k]; p++) {
                Li[nz] = k1 + lu->Li[lu->Lip[k] + p];
                Lx[nz] = lu->Lx[lu->Lip[k] + p];
                nz++;
            }
        }
    }
    Lp[n] = nz;
    nz = 0;
    for (int b = 0; b < lu->nblocks; b++) {
        int k1 = lu->R[b], k2 = lu->R[b + 1];
        for (int k = k1; k < k2; k++) {
            Up[k] = nz;
            for (int p = 0; p < lu->Ulen[k]; p++) {
                Ui[nz] = k1 + lu->Ui[lu->Uip[k] + p];
                Ux[nz] = lu->Ux[lu->Uip[k] + p];
                nz++;
            }
            Ui[nz] = k; Ux[nz] = lu->Udiag[k]; nz++;
        }
    }
    Up[n] = nz;
    for (int k = 0; k <= n; k++) Fp[k] = lu->Offp[k];
    for (int p = 0; p < lu->nzoff; p++) { Fi[p] = lu->Offi[p]; Fx[p] = lu->Offx[p]; }
    for (int k = 0; k < n; k++) { Pnum[k] = lu->Pnum[k]; Q[k] = lu->Q[k]; }
    for (int b = 0; b <= lu->nblocks; b++) R[b] = lu->R[b];
}

/* ------------------------------------------------------------------------ */
/* Topology + newton_raphson_cached (src/solver.rs:639-736)                  */

struct gxo_topo {
    int n, nnzy;
    int32_t *yp, *yi, *bus_type;
    double *yre, *yim;
    gxo_jac *jac;
    int32_t *P, *Q, *R;
    int nblocks;
    int32_t *ns_idx, *pq_idx;
    int n_ang, n_pq;
    double *zip; /* NULL, or [4][n]: impedance re, im; current re, im (per unit at |V| = 1) */
};

gxo_topo *gxo_topo_new(int n, const int32_t *yp, const int32_t *yi, const double *yre,
                       const double *yim, const int32_t *bus_type, const int32_t *P,
                       const int32_t *Q, const int32_t *R, int nblocks) {
    gxo_topo *t = (gxo_topo *)xcalloc(1, sizeof(gxo_topo));
    int nnz = yp[n];
    t->n = n;
    t->nnzy = nnz;
    t->yp = (int32_t *)xmalloc(sizeof(int32_t) * (n + 1));
    t->yi = (int32_t *)xmalloc(sizeof(int32_t) * nnz);
    t->yre = (double *)xmalloc(sizeof(double) * nnz);
    t->yim = (double *)xmalloc(sizeof(double) * nnz);
    t->bus_type = (int32_t *)xmalloc(sizeof(int32_t) * n);
    memcpy(t->yp, yp, sizeof(int32_t) * (n + 1));
    memcpy(t->yi, yi, sizeof(int32_t) * nnz);
    memcpy(t->yre, yre, sizeof(double) * nnz);
    memcpy(t->yim, yim, sizeof(double) * nnz);
    memcpy(t->bus_type, bus_type, sizeof(int32_t) * n);
    t->jac = gxo_jac_analyze(n, yp, yi, bus_type);
    int nu = t->jac->n_u;
    t->P = (int32_t *)xmalloc(sizeof(int32_t) * (nu + 1));
    t->Q = (int32_t *)xmalloc(sizeof(int32_t) * (nu + 1));
    t->R = (int32_t *)xmalloc(sizeof(int32_t) * (nblocks + 1));
    memcpy(t->P, P, sizeof(int32_t) * nu);
    memcpy(t->Q, Q, sizeof(int32_t) * nu);
    memcpy(t->R, R, sizeof(int32_t) * (nblocks + 1));
    t->nblocks = nblocks;
    t->ns_idx = (int32_t *)xmalloc(sizeof(int32_t) * n);
    t->pq_idx = (int32_t *)xmalloc(sizeof(int32_t) * n);
    for (int i = 0; i < n; i++) {
        if (bus_type[i] != GXO_SLACK) t->ns_idx[t->n_ang++] = i;
    }
    for (int i = 0; i < n; i++) {
        if (bus_type[i] == GXO_PQ) t->pq_idx[t->n_pq++] = i;
    }
    return t;
}

/* ZIP terms of effective_injection (src/network.rs:600-611): per bus one
 * constant-impedance and one constant-current term (each the sum of the bus's
 * terms of that kind); NULL clears them. */
void gxo_topo_set_zip(gxo_topo *t, const double *zi_re, const double *zi_im, const double *zc_re,
                      const double *zc_im) {
    free(t->zip);
    t->zip = NULL;
    if (!zi_re) return;
    t->zip = (double *)xmalloc(sizeof(double) * 4 * (size_t)t->n);
    memcpy(t->zip, zi_re, sizeof(double) * t->n);
    memcpy(t->zip + t->n, zi_im, sizeof(double) * t->n);
    memcpy(t->zip + 2 * t->n, zc_re, sizeof(double) * t->n);
    memcpy(t->zip + 3 * t->n, zc_im, sizeof(double) * t->n);
}

/* effective_injection (src/network.rs:600-611): s = p + jq; s += s_imp * |V|
 * * |V| (constant impedance); s += s_cur * |V| (constant current). */
static double eff_p(const gxo_topo *t, int i, double p, double vm) {
    if (!t->zip) return p;
    double s = p;
    s += t->zip[i] * vm * vm;
    s += t->zip[2 * t->n + i] * vm;
    return s;
}
static double eff_q(const gxo_topo *t, int i, double q, double vm) {
    if (!t->zip) return q;
    double s = q;
    s += t->zip[t->n + i] * vm * vm;
    s += t->zip[3 * t->n + i] * vm;
    return s;
}

void gxo_topo_free(gxo_topo *t) {
    if (!t) return;
    free(t->zip);
    free(t->yp); free(t->yi); free(t->yre); free(t->yim); free(t->bus_type);
    gxo_jac_free(t->jac);
    free(t->P); free(t->Q); free(t->R); free(t->ns_idx); free(t->pq_idx);
    free(t);
}

int gxo_nr_solve(gxo_topo *t, gxo_lu **cache, const double *yre, const double *yim,
                 double *vm, double *va, const double *p_spec, const double *q_spec,
                 double tol, int max_iter, double *hist, int *iters) {
    int n = t->n, nu = t->jac->n_u, nnzj = t->jac->nnz;
    if (!yre) yre = t->yre;
    if (!yim) yim = t->yim;
    double *p = (double *)xmalloc(sizeof(double) * n);
    double *q = (double *)xmalloc(sizeof(double) * n);
    double *mis = (double *)xmalloc(sizeof(double) * (nu + 1));
    double *dx = (double *)xmalloc(sizeof(double) * (nu + 1));
    double *vals = (double *)xmalloc(sizeof(double) * (nnzj + 1));
    int status = GXO_MAXITER, it;
    *iters = 0;
    for (it = 0; it < max_iter; it++) {
        gxo_injections(n, t->yp, t->yi, yre, yim, vm, va, p, q);
        int m = 0;
        for (int a = 0; a < t->n_ang; a++) {
            int i = t->ns_idx[a];
            mis[m++] = eff_p(t, i, p_spec[i], vm[i]) - p[i];
        }
        for (int a = 0; a < t->n_pq; a++) {
            int i = t->pq_idx[a];
            mis[m++] = eff_q(t, i, q_spec[i], vm[i]) - q[i];
        }
        /* fold(0.0, |a, b| a.max(b.abs())); f64::max and fmax both skip NaN */
        double mx = 0.0;
        for (int a = 0; a < nu; a++) mx = fmax(mx, fabs(mis[a]));
        if (hist) hist[it] = mx;
        *iters = it + 1;
        if (mx < tol) { status = GXO_CONVERGED; break; }
        gxo_jac_fill(t->jac, yre, yim, vm, va, p, q, vals);
        if (!*cache) {
            int st;
            *cache = gxo_lu_new(nu, nnzj, t->jac->rows, t->jac->cols, vals, t->P, t->Q, t->R,
                                t->nblocks, &st);
            if (!*cache) { status = GXO_SINGULAR; break; }
        }
        if (gxo_lu_factor_solve_values(*cache, vals, mis, dx)) { status = GXO_SINGULAR; break; }
        int d = 0;
        for (int a = 0; a < t->n_ang; a++) va[t->ns_idx[a]] += dx[d++];
        for (int a = 0; a < t->n_pq; a++) vm[t->pq_idx[a]] += dx[d++];
    }
    free(p); free(q); free(mis); free(dx); free(vals);
    return status;
}

/* ------------------------------------------------------------------------ */
/* BatchSolver::solve (src/batch.rs:198-289)                                 */

typedef struct {
    gxo_topo *t;
    int B;
    const double *p_spec, *q_spec, *vm0, *va0, *dre, *dim;
    int v_stride;
    const int32_t *dslot;
    double tol;
    int max_iter;
    double *vm_out, *va_out, *max_mis, *hist;
    int32_t *iters, *status;
    int next; /* shared work counter */
    pthread_mutex_t mu;
} batch_job;

static void *batch_worker(void *arg) {
    batch_job *J = (batch_job *)arg;
    gxo_topo *t = J->t;
    int n = t->n;
    gxo_lu *cache = NULL; /* one persistent solver per worker (batch.rs:246) */
    double *yre = NULL, *yim = NULL;
    double *h = (double *)xmalloc(sizeof(double) * (J->max_iter + 1));
    if (J->dslot) {
        yre = (double *)xmalloc(sizeof(double) * t->nnzy);
        yim = (double *)xmalloc(sizeof(double) * t->nnzy);
    }
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int s = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (s >= J->B) break;
        double *vm = J->vm_out + (size_t)s * n;
        double *va = J->va_out + (size_t)s * n;
        memcpy(vm, J->vm0 + (size_t)s * J->v_stride, sizeof(double) * n);
        memcpy(va, J->va0 + (size_t)s * J->v_stride, sizeof(double) * n);
        const double *yr = t->yre, *yi = t->yim;
        if (J->dslot) {
            memcpy(yre, t->yre, sizeof(double) * t->nnzy);
            memcpy(yim, t->yim, sizeof(double) * t->nnzy);
            for (int c = 0; c < 4; c++) {
                int sl = J->dslot[(size_t)s * 4 + c];
                yre[sl] += J->dre[(size_t)s * 4 + c];
                yim[sl] += J->dim[(size_t)s * 4 + c];
            }
            yr = yre;
            yi = yim;
        }
        int it = 0;
        int st = gxo_nr_solve(t, &cache, yr, yi, vm, va, J->p_spec + (size_t)s * n,
                              J->q_spec + (size_t)s * n, J->tol, J->max_iter, h, &it);
        J->iters[s] = it;
        J->status[s] = st;
        J->max_mis[s] = it > 0 ? h[it - 1] : 0.0;
        if (J->hist) {
            for (int k = 0; k < J->max_iter; k++)
                J->hist[(size_t)s * J->max_iter + k] = k < it ? h[k] : 0.0;
        }
    }
    gxo_lu_free(cache);
    free(h);
    free(yre);
    free(yim);
    return NULL;
}

int gxo_batch_solve(gxo_topo *t, int B, const double *p_spec, const double *q_spec,
                    const double *vm0, const double *va0, int v_stride, const int32_t *dslot,
                    const double *dre, const double *dim, double tol, int max_iter,
                    int nthreads, double *vm_out, double *va_out, int32_t *iters,
                    int32_t *status, double *max_mis, double *hist) {
    if (B <= 0) return 0;
    batch_job J;
    memset(&J, 0, sizeof(J));
    J.t = t; J.B = B; J.p_spec = p_spec; J.q_spec = q_spec; J.vm0 = vm0; J.va0 = va0;
    J.v_stride = v_stride; J.dslot = dslot; J.dre = dre; J.dim = dim; J.tol = tol;
    J.max_iter = max_iter; J.vm_out = vm_out; J.va_out = va_out; J.iters = iters;
    J.status = status; J.max_mis = max_mis; J.hist = hist;
    pthread_mutex_init(&J.mu, NULL);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > B) nthreads = B;
    /* every worker, a single one included, runs on a thread of its own: the
       calling thread's allocator arena behaves differently (on the Arm host
       it ran one worker 2.7x slower), and a thread count of 1 must measure
       the same worker as the others */
    pthread_t *th = (pthread_t *)xmalloc(sizeof(pthread_t) * nthreads);
    for (int w = 0; w < nthreads; w++) pthread_create(&th[w], NULL, batch_worker, &J);
    for (int w = 0; w < nthreads; w++) pthread_join(th[w], NULL);
    free(th);
    pthread_mutex_destroy(&J.mu);
    return 0;
}
