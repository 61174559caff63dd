// Host symbolic analysis: Jacobian pattern, CSC map, BTF, AMD, first factor.
// See gox_symbolic.hpp.  Each routine follows the reference step for step
// where its output must be identical (orderings, pivot rows, patterns); the
// file:line each one follows is given at the routine.
//
// Provenance and licences.  The ordering and first-factor routines restate
// SuiteSparse (v7.12.2) closely, because their outputs must equal KLU's bit
// for bit, so they carry the upstream packages' notices:
//   * btf_maxtrans, btf_strongcomp, btf_order -- from BTF/Source/btf_*.c:
//       BTF, Copyright (c) 2004-2022, University of Florida.  All Rights Reserved.
//       SPDX-License-Identifier: LGPL-2.1+
//   * clear_w, amd_postorder, amd_eliminate, amd_order -- from
//     AMD/Source/amd_{order,aat,1,2,postorder,post_tree}.c:
//       AMD, Copyright (c) 1996-2022, Timothy A. Davis, Patrick R. Amestoy,
//       and Iain S. Duff.  All Rights Reserved.
//       SPDX-License-Identifier: BSD-3-clause
//   * klu_analyze, klu_factor -- from KLU/Source/klu_analyze.c, klu_factor.c,
//     klu_kernel.c:
//       KLU, Copyright (c) 2004-2022, University of Florida.  All Rights Reserved.
//       SPDX-License-Identifier: LGPL-2.1+
// jac_analyze and build_csc restate the reference's own Rust
// (src/jacobian.rs, src/klu_native/mod.rs).  libgridoxide_gb300.so therefore
// contains code derived from LGPL-2.1+ sources (BTF, KLU).
#include "gox_symbolic.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>

namespace gox {

static constexpr int32_t EMPTY = -1;
static inline int32_t flip(int32_t i) { return -i - 2; }
static inline int32_t unflip(int32_t i) { return i < EMPTY ? flip(i) : i; }

// ---------------------------------------------------------------------------
// JacobianPattern::analyze (src/jacobian.rs:96-171)

JacPattern jac_analyze(int n, const int32_t* yp, const int32_t* yi, const int32_t* bus_type) {
  JacPattern J;
  J.n_bus = n;
  J.ns_pos.assign(n, -1);
  J.pq_pos.assign(n, -1);
  for (int i = 0; i < n; i++)
    if (bus_type[i] != BUS_SLACK) { J.ns_pos[i] = J.n_ang++; J.ns_idx.push_back(i); }
  for (int i = 0; i < n; i++)
    if (bus_type[i] == BUS_PQ) { J.pq_pos[i] = J.n_pq++; J.pq_idx.push_back(i); }
  J.n_u = J.n_ang + J.n_pq;
  auto push = [&](int r, int c, int k, int i, int kk, int s) {
    J.rows.push_back(r); J.cols.push_back(c); J.kind.push_back(k);
    J.bi.push_back(i); J.bk.push_back(kk); J.yslot.push_back(s);
  };
  for (int i = 0; i < n; i++) {  // H and N rows
    if (J.ns_pos[i] < 0) continue;
    int row = J.ns_pos[i];
    for (int s = yp[i]; s < yp[i + 1]; s++) {
      int k = yi[s];
      if (k == i) {
        push(row, row, K_HII, i, i, s);
        if (J.pq_pos[i] >= 0) push(row, J.n_ang + J.pq_pos[i], K_NII, i, i, s);
        continue;
      }
      if (J.ns_pos[k] >= 0) push(row, J.ns_pos[k], K_HIK, i, k, s);
      if (J.pq_pos[k] >= 0) push(row, J.n_ang + J.pq_pos[k], K_NIK, i, k, s);
    }
  }
  for (int i = 0; i < n; i++) {  // M and L rows
    if (J.pq_pos[i] < 0) continue;
    int row = J.n_ang + J.pq_pos[i];
    for (int s = yp[i]; s < yp[i + 1]; s++) {
      int k = yi[s];
      if (k == i) {
        push(row, J.ns_pos[i], K_MII, i, i, s);
        push(row, row, K_LII, i, i, s);
        continue;
      }
      if (J.ns_pos[k] >= 0) push(row, J.ns_pos[k], K_MIK, i, k, s);
      if (J.pq_pos[k] >= 0) push(row, J.n_ang + J.pq_pos[k], K_LIK, i, k, s);
    }
  }
  return J;
}

// ---------------------------------------------------------------------------
// build_csc_structure (src/klu_native/mod.rs:88-114)

Csc build_csc(int n, int nt, const int32_t* rows, const int32_t* cols) {
  Csc A;
  A.n = n;
  std::vector<int32_t> order(nt);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (cols[a] != cols[b]) return cols[a] < cols[b];
    return rows[a] < rows[b];
  });
  A.p.assign(n + 1, 0);
  A.slot_of.assign(nt, -1);
  for (int idx = 0; idx < nt;) {
    int r = rows[order[idx]], c = cols[order[idx]];
    int s = (int)A.i.size();
    A.i.push_back(r);
    A.p[c + 1]++;
    while (idx < nt && rows[order[idx]] == r && cols[order[idx]] == c) A.slot_of[order[idx++]] = s;
  }
  for (int c = 0; c < n; c++) A.p[c + 1] += A.p[c];
  return A;
}

// ---------------------------------------------------------------------------
// BTF maximum transversal (BTF/Source/btf_maxtrans.c: depth-first augmenting
// paths with a cheap-assignment pointer per column; no work limit).

int btf_maxtrans(int n, const int32_t* Ap, const int32_t* Ai, int32_t* match) {
  std::vector<int32_t> cheap(Ap, Ap + n), flag(n, EMPTY), istack(n), jstack(n), pstack(n);
  for (int i = 0; i < n; i++) match[i] = EMPTY;
  int nmatch = 0;
  for (int k = 0; k < n; k++) {
    bool found = false;
    int i = EMPTY, head = 0;
    jstack[0] = k;
    while (head >= 0) {
      int j = jstack[head];
      int pend = Ap[j + 1];
      if (flag[j] != k) {  // first visit: cheap test for an unmatched row
        flag[j] = k;
        int p;
        for (p = cheap[j]; p < pend && !found; p++) {
          i = Ai[p];
          found = (match[i] == EMPTY);
        }
        cheap[j] = p;
        if (found) { istack[head] = i; break; }
        pstack[head] = Ap[j];
      }
      int p;
      for (p = pstack[head]; p < pend; p++) {  // depth-first through matched rows
        i = Ai[p];
        int j2 = match[i];
        if (flag[j2] != k) {
          pstack[head] = p + 1;
          istack[head] = i;
          jstack[++head] = j2;
          break;
        }
      }
      if (p == pend) head--;
    }
    if (found) {
      for (int p = head; p >= 0; p--) match[istack[p]] = jstack[p];
      nmatch++;
    }
  }
  return nmatch;
}

// Tarjan strongly connected components on the matched graph
// (BTF/Source/btf_strongcomp.c, non-recursive variant).
int btf_strongcomp(int n, const int32_t* Ap, const int32_t* Ai, int32_t* Q, int32_t* P,
                   int32_t* R) {
  const int32_t UNVISITED = -2, UNASSIGNED = -1;
  std::vector<int32_t> time(n, EMPTY), flag(n, UNVISITED), low(n, EMPTY), cstack(n + 1),
      jstack(n), pstack(n);
  int timestamp = 0, nblocks = 0;
  for (int j0 = 0; j0 < n; j0++) {
    if (flag[j0] != UNVISITED) continue;
    int chead = 0, jhead = 0;
    jstack[0] = j0;
    while (jhead >= 0) {
      int j = jstack[jhead];
      int jj = Q ? unflip(Q[j]) : j;
      int pend = Ap[jj + 1];
      if (flag[j] == UNVISITED) {
        cstack[++chead] = j;
        timestamp++;
        time[j] = timestamp;
        low[j] = timestamp;
        flag[j] = UNASSIGNED;
        pstack[jhead] = Ap[jj];
      }
      int p;
      for (p = pstack[jhead]; p < pend; p++) {
        int i = Ai[p];
        if (flag[i] == UNVISITED) {
          pstack[jhead] = p + 1;
          jstack[++jhead] = i;
          break;
        } else if (flag[i] == UNASSIGNED) {
          low[j] = std::min(low[j], time[i]);
        }
      }
      if (p == pend) {
        jhead--;
        if (low[j] == time[j]) {
          for (;;) {
            int i = cstack[chead--];
            flag[i] = nblocks;
            if (i == j) break;
          }
          nblocks++;
        }
        if (jhead >= 0) {
          int parent = jstack[jhead];
          low[parent] = std::min(low[parent], low[j]);
        }
      }
    }
  }
  std::vector<int32_t> cnt(nblocks + 1, 0), start(nblocks + 1, 0);
  for (int j = 0; j < n; j++) cnt[flag[j]]++;
  for (int b = 1; b < nblocks; b++) start[b] = start[b - 1] + cnt[b - 1];
  for (int b = 0; b < nblocks; b++) R[b] = start[b];
  R[nblocks] = n;
  for (int j = 0; j < n; j++) P[start[flag[j]]++] = j;
  if (Q) {
    std::vector<int32_t> qn(n);
    for (int k = 0; k < n; k++) qn[k] = Q[P[k]];
    std::copy(qn.begin(), qn.end(), Q);
  }
  return nblocks;
}

// btf_order (BTF/Source/btf_order.c): matching, complete it for structurally
// singular matrices (unmatched columns, highest first, flipped), then SCC.
int btf_order(int n, const int32_t* Ap, const int32_t* Ai, int32_t* P, int32_t* Q, int32_t* R,
              int* nmatch) {
  *nmatch = btf_maxtrans(n, Ap, Ai, Q);
  if (*nmatch < n) {
    std::vector<char> used(n, 0);
    for (int i = 0; i < n; i++)
      if (Q[i] != EMPTY) used[Q[i]] = 1;
    std::vector<int32_t> bad;
    for (int j = n - 1; j >= 0; j--)
      if (!used[j]) bad.push_back(j);
    for (int i = 0; i < n; i++)
      if (Q[i] == EMPTY && !bad.empty()) { Q[i] = flip(bad.back()); bad.pop_back(); }
  }
  return btf_strongcomp(n, Ap, Ai, Q, P, R);
}

// ---------------------------------------------------------------------------
// AMD (AMD/Source/amd_order.c, amd_aat.c, amd_1.c, amd_2.c, amd_postorder.c,
// amd_post_tree.c).  The quotient-graph elimination keeps the reference's
// in-place list layout (one workspace array with per-variable offsets and
// the in-place garbage collection), because the order of entries inside
// each list decides ties between equal degrees and so the permutation.

namespace {

struct AmdWork {
  int n;
  std::vector<int32_t> Pe, Nv, Next, Last, Head, Elen, Degree, W, Len, Iw;
  int iwlen, pfree;
};

int32_t clear_w(int32_t wflg, int32_t wbig, std::vector<int32_t>& W, int n) {
  if (wflg < 2 || wflg >= wbig) {
    for (int x = 0; x < n; x++)
      if (W[x] != 0) W[x] = 1;
    wflg = 2;
  }
  return wflg;
}

// Depth-first postorder of the assembly tree; the child with the largest
// front goes last among its siblings.
void amd_postorder(int n, const int32_t* parent, const int32_t* nv, const int32_t* fsize,
                   int32_t* order) {
  std::vector<int32_t> child(n, EMPTY), sibling(n, EMPTY), stack(n);
  for (int j = n - 1; j >= 0; j--) {
    if (nv[j] > 0 && parent[j] != EMPTY) {
      sibling[j] = child[parent[j]];
      child[parent[j]] = j;
    }
  }
  for (int i = 0; i < n; i++) {
    if (nv[i] > 0 && child[i] != EMPTY) {
      int fprev = EMPTY, maxfrsize = EMPTY, bigfprev = EMPTY, bigf = EMPTY;
      for (int f = child[i]; f != EMPTY; f = sibling[f]) {
        if (fsize[f] >= maxfrsize) { maxfrsize = fsize[f]; bigfprev = fprev; bigf = f; }
        fprev = f;
      }
      int fnext = sibling[bigf];
      if (fnext != EMPTY) {
        if (bigfprev == EMPTY) child[i] = fnext; else sibling[bigfprev] = fnext;
        sibling[bigf] = EMPTY;
        sibling[fprev] = bigf;
      }
    }
  }
  for (int i = 0; i < n; i++) order[i] = EMPTY;
  int k = 0;
  for (int root = 0; root < n; root++) {
    if (parent[root] != EMPTY || nv[root] <= 0) continue;
    int head = 0;
    stack[0] = root;
    while (head >= 0) {
      int i = stack[head];
      if (child[i] != EMPTY) {
        for (int f = child[i]; f != EMPTY; f = sibling[f]) head++;
        int h = head;
        for (int f = child[i]; f != EMPTY; f = sibling[f]) stack[h--] = f;
        child[i] = EMPTY;
      } else {
        head--;
        order[i] = k++;
      }
    }
  }
}

// The elimination proper (amd_2.c): returns Last = permutation.
void amd_eliminate(AmdWork& A, int32_t* Last_out) {
  const int n = A.n;
  auto& Pe = A.Pe; auto& Nv = A.Nv; auto& Next = A.Next; auto& Last = A.Last;
  auto& Head = A.Head; auto& Elen = A.Elen; auto& Degree = A.Degree; auto& W = A.W;
  auto& Len = A.Len; auto& Iw = A.Iw;
  int iwlen = A.iwlen, pfree = A.pfree;

  int dense = (int)(10.0 * std::sqrt((double)n));
  dense = std::max(16, dense);
  dense = std::min(n, dense);
  for (int i = 0; i < n; i++) {
    Last[i] = EMPTY; Head[i] = EMPTY; Next[i] = EMPTY;
    Nv[i] = 1; W[i] = 1; Elen[i] = 0; Degree[i] = Len[i];
  }
  const int32_t wbig = std::numeric_limits<int32_t>::max() - n;
  int32_t wflg = clear_w(0, wbig, W, n);
  int nel = 0, mindeg = 0, lemax = 0;

  // initial degree lists; empty rows become elements, dense rows go last
  for (int i = 0; i < n; i++) {
    int deg = Degree[i];
    if (deg == 0) {
      Elen[i] = flip(1); nel++; Pe[i] = EMPTY; W[i] = 0;
    } else if (deg > dense) {
      Nv[i] = 0; Elen[i] = EMPTY; nel++; Pe[i] = EMPTY;
    } else {
      int inext = Head[deg];
      if (inext != EMPTY) Last[inext] = i;
      Next[i] = inext;
      Head[deg] = i;
    }
  }

  auto unlink_degree = [&](int i) {
    int ilast = Last[i], inext = Next[i];
    if (inext != EMPTY) Last[inext] = ilast;
    if (ilast != EMPTY) Next[ilast] = inext; else Head[Degree[i]] = inext;
  };

  while (nel < n) {
    // -- pivot of minimum approximate degree
    int deg, me = EMPTY;
    for (deg = mindeg; deg < n; deg++) {
      me = Head[deg];
      if (me != EMPTY) break;
    }
    mindeg = deg;
    {
      int inext = Next[me];
      if (inext != EMPTY) Last[inext] = EMPTY;
      Head[deg] = inext;
    }
    int elenme = Elen[me];
    int nvpiv = Nv[me];
    nel += nvpiv;
    Nv[me] = -nvpiv;
    int degme = 0;
    int pme1, pme2;

    // -- construct the new element Lme
    if (elenme == 0) {
      pme1 = Pe[me];
      pme2 = pme1 - 1;
      for (int p = pme1; p <= pme1 + Len[me] - 1; p++) {
        int i = Iw[p];
        int nvi = Nv[i];
        if (nvi > 0) {
          degme += nvi;
          Nv[i] = -nvi;
          Iw[++pme2] = i;
          unlink_degree(i);
        }
      }
    } else {
      int p = Pe[me];
      pme1 = pfree;
      int slenme = Len[me] - elenme;
      for (int knt1 = 1; knt1 <= elenme + 1; knt1++) {
        int e, pj, ln;
        if (knt1 > elenme) { e = me; pj = p; ln = slenme; }
        else { e = Iw[p++]; pj = Pe[e]; ln = Len[e]; }
        for (int knt2 = 1; knt2 <= ln; knt2++) {
          int i = Iw[pj++];
          int nvi = Nv[i];
          if (nvi <= 0) continue;
          if (pfree >= iwlen) {
            // compress Iw in place (garbage collection)
            Pe[me] = p;
            Len[me] -= knt1;
            if (Len[me] == 0) Pe[me] = EMPTY;
            Pe[e] = pj;
            Len[e] = ln - knt2;
            if (Len[e] == 0) Pe[e] = EMPTY;
            for (int j = 0; j < n; j++) {
              int pn = Pe[j];
              if (pn >= 0) { Pe[j] = Iw[pn]; Iw[pn] = flip(j); }
            }
            int psrc = 0, pdst = 0, pend = pme1 - 1;
            while (psrc <= pend) {
              int j = flip(Iw[psrc++]);
              if (j >= 0) {
                Iw[pdst] = Pe[j];
                Pe[j] = pdst++;
                int lenj = Len[j];
                for (int knt3 = 0; knt3 <= lenj - 2; knt3++) Iw[pdst++] = Iw[psrc++];
              }
            }
            int p1 = pdst;
            for (psrc = pme1; psrc <= pfree - 1; psrc++) Iw[pdst++] = Iw[psrc];
            pme1 = p1;
            pfree = pdst;
            pj = Pe[e];
            p = Pe[me];
          }
          degme += nvi;
          Nv[i] = -nvi;
          Iw[pfree++] = i;
          unlink_degree(i);
        }
        if (e != me) { Pe[e] = flip(me); W[e] = 0; }  // absorb e into me
      }
      pme2 = pfree - 1;
    }
    Degree[me] = degme;
    Pe[me] = pme1;
    Len[me] = pme2 - pme1 + 1;
    Elen[me] = flip(nvpiv + degme);

    // -- scan 1: |Le \ Lme| for every element e adjacent to Lme
    wflg = clear_w(wflg, wbig, W, n);
    for (int pme = pme1; pme <= pme2; pme++) {
      int i = Iw[pme];
      int eln = Elen[i];
      if (eln <= 0) continue;
      int nvi = -Nv[i];
      int wnvi = wflg - nvi;
      for (int p = Pe[i]; p <= Pe[i] + eln - 1; p++) {
        int e = Iw[p];
        int we = W[e];
        if (we >= wflg) we -= nvi;
        else if (we != 0) we = Degree[e] + wnvi;
        W[e] = we;
      }
    }

    // -- scan 2: degree update, element absorption, hashing
    for (int pme = pme1; pme <= pme2; pme++) {
      int i = Iw[pme];
      int p1 = Pe[i];
      int p2 = p1 + Elen[i] - 1;
      int pn = p1;
      uint32_t hash = 0;
      int dg = 0;
      for (int p = p1; p <= p2; p++) {  // aggressive absorption on
        int e = Iw[p];
        int we = W[e];
        if (we == 0) continue;
        int dext = we - wflg;
        if (dext > 0) {
          dg += dext;
          Iw[pn++] = e;
          hash += (uint32_t)e;
        } else {
          Pe[e] = flip(me);
          W[e] = 0;
        }
      }
      Elen[i] = pn - p1 + 1;
      int p3 = pn;
      int p4 = p1 + Len[i];
      for (int p = p2 + 1; p < p4; p++) {
        int j = Iw[p];
        int nvj = Nv[j];
        if (nvj > 0) {
          dg += nvj;
          Iw[pn++] = j;
          hash += (uint32_t)j;
        }
      }
      if (Elen[i] == 1 && p3 == pn) {  // mass elimination
        Pe[i] = flip(me);
        int nvi = -Nv[i];
        degme -= nvi;
        nvpiv += nvi;
        nel += nvi;
        Nv[i] = 0;
        Elen[i] = EMPTY;
      } else {
        Degree[i] = std::min(Degree[i], dg);
        Iw[pn] = Iw[p3];
        Iw[p3] = Iw[p1];
        Iw[p1] = me;
        Len[i] = pn - p1 + 1;
        int h = (int)(hash % (uint32_t)n);
        int j = Head[h];
        if (j <= EMPTY) { Next[i] = flip(j); Head[h] = flip(i); }
        else { Next[i] = Last[j]; Last[j] = i; }
        Last[i] = h;
      }
    }
    Degree[me] = degme;
    lemax = std::max(lemax, degme);
    wflg += lemax;
    wflg = clear_w(wflg, wbig, W, n);

    // -- supervariable detection
    for (int pme = pme1; pme <= pme2; pme++) {
      int i = Iw[pme];
      if (Nv[i] >= 0) continue;
      int h = Last[i];
      int j = Head[h];
      if (j == EMPTY) i = EMPTY;
      else if (j < EMPTY) { i = flip(j); Head[h] = EMPTY; }
      else { i = Last[j]; Last[j] = EMPTY; }
      while (i != EMPTY && Next[i] != EMPTY) {
        int ln = Len[i], eln = Elen[i];
        for (int p = Pe[i] + 1; p <= Pe[i] + ln - 1; p++) W[Iw[p]] = wflg;
        int jlast = i;
        j = Next[i];
        while (j != EMPTY) {
          bool ok = (Len[j] == ln) && (Elen[j] == eln);
          for (int p = Pe[j] + 1; ok && p <= Pe[j] + ln - 1; p++)
            if (W[Iw[p]] != wflg) ok = false;
          if (ok) {
            Pe[j] = flip(i);
            Nv[i] += Nv[j];
            Nv[j] = 0;
            Elen[j] = EMPTY;
            j = Next[j];
            Next[jlast] = j;
          } else {
            jlast = j;
            j = Next[j];
          }
        }
        wflg++;
        i = Next[i];
      }
    }

    // -- finalize Lme, restore degree lists
    int p = pme1;
    int nleft = n - nel;
    for (int pme = pme1; pme <= pme2; pme++) {
      int i = Iw[pme];
      int nvi = -Nv[i];
      if (nvi <= 0) continue;
      Nv[i] = nvi;
      int dg = Degree[i] + degme - nvi;
      dg = std::min(dg, nleft - nvi);
      int inext = Head[dg];
      if (inext != EMPTY) Last[inext] = i;
      Next[i] = inext;
      Last[i] = EMPTY;
      Head[dg] = i;
      mindeg = std::min(mindeg, dg);
      Degree[i] = dg;
      Iw[p++] = i;
    }
    Nv[me] = nvpiv;
    Len[me] = p - pme1;
    if (Len[me] == 0) { Pe[me] = EMPTY; W[me] = 0; }
    if (elenme != 0) pfree = p;
  }

  // -- assembly tree, postorder, permutation
  for (int i = 0; i < n; i++) Pe[i] = flip(Pe[i]);
  for (int i = 0; i < n; i++) Elen[i] = flip(Elen[i]);
  for (int i = 0; i < n; i++) {
    if (Nv[i] != 0) continue;
    int j = Pe[i];
    if (j == EMPTY) continue;
    while (Nv[j] == 0) j = Pe[j];
    int e = j;
    j = i;
    while (Nv[j] == 0) {
      int jnext = Pe[j];
      Pe[j] = e;
      j = jnext;
    }
  }
  amd_postorder(n, Pe.data(), Nv.data(), Elen.data(), W.data());
  for (int k = 0; k < n; k++) { Head[k] = EMPTY; Next[k] = EMPTY; }
  for (int e = 0; e < n; e++) {
    int k = W[e];
    if (k != EMPTY) Head[k] = e;
  }
  int nel2 = 0;
  for (int k = 0; k < n; k++) {
    int e = Head[k];
    if (e == EMPTY) break;
    Next[e] = nel2;
    nel2 += Nv[e];
  }
  for (int i = 0; i < n; i++) {
    if (Nv[i] != 0) continue;
    int e = Pe[i];
    if (e != EMPTY) { Next[i] = Next[e]; Next[e]++; }
    else Next[i] = nel2++;
  }
  for (int i = 0; i < n; i++) Last_out[Next[i]] = i;
}

}  // namespace

int amd_order(int n, const int32_t* Ap_in, const int32_t* Ai_in, int32_t* perm) {
  if (n == 0) return 0;
  // validity / jumbled check (amd_valid.c)
  if (Ap_in[0] != 0 || Ap_in[n] < 0) return -1;
  bool jumbled = false;
  for (int j = 0; j < n; j++) {
    if (Ap_in[j] > Ap_in[j + 1]) return -1;
    int ilast = EMPTY;
    for (int p = Ap_in[j]; p < Ap_in[j + 1]; p++) {
      int i = Ai_in[p];
      if (i < 0 || i >= n) return -1;
      if (i <= ilast) jumbled = true;
      ilast = i;
    }
  }
  // jumbled input is replaced by its sorted, duplicate-free transpose
  // (amd_preprocess.c)
  std::vector<int32_t> Rp, Ri;
  const int32_t* Ap = Ap_in;
  const int32_t* Ai = Ai_in;
  if (jumbled) {
    std::vector<int32_t> w(n, 0), flag(n, EMPTY);
    for (int j = 0; j < n; j++)
      for (int p = Ap_in[j]; p < Ap_in[j + 1]; p++) {
        int i = Ai_in[p];
        if (flag[i] != j) { w[i]++; flag[i] = j; }
      }
    Rp.assign(n + 1, 0);
    for (int i = 0; i < n; i++) Rp[i + 1] = Rp[i] + w[i];
    Ri.assign(std::max(Rp[n], 1), 0);
    for (int i = 0; i < n; i++) { w[i] = Rp[i]; flag[i] = EMPTY; }
    for (int j = 0; j < n; j++)
      for (int p = Ap_in[j]; p < Ap_in[j + 1]; p++) {
        int i = Ai_in[p];
        if (flag[i] != j) { Ri[w[i]++] = j; flag[i] = j; }
      }
    Ap = Rp.data();
    Ai = Ri.data();
  }
  // |A + A'| per column, diagonal excluded (amd_aat.c)
  AmdWork A;
  A.n = n;
  A.Len.assign(n, 0);
  std::vector<int32_t> Tp(n, 0);
  for (int k = 0; k < n; k++) {
    int p;
    for (p = Ap[k]; p < Ap[k + 1];) {
      int j = Ai[p];
      if (j < k) { A.Len[j]++; A.Len[k]++; p++; }
      else if (j == k) { p++; break; }
      else break;
      int pj;
      for (pj = Tp[j]; pj < Ap[j + 1];) {
        int i = Ai[pj];
        if (i < k) { A.Len[i]++; A.Len[j]++; pj++; }
        else if (i == k) { pj++; break; }
        else break;
      }
      Tp[j] = pj;
    }
    Tp[k] = p;
  }
  for (int j = 0; j < n; j++)
    for (int pj = Tp[j]; pj < Ap[j + 1]; pj++) { A.Len[Ai[pj]]++; A.Len[j]++; }
  size_t nzaat = 0;
  for (int k = 0; k < n; k++) nzaat += A.Len[k];
  size_t slen = nzaat + nzaat / 5 + 7 * (size_t)n;
  A.iwlen = (int)(slen - 6 * (size_t)n);
  A.Iw.assign(A.iwlen, 0);
  A.Pe.assign(n, 0); A.Nv.assign(n, 0); A.Next.assign(n, 0); A.Last.assign(n, 0);
  A.Head.assign(n, 0); A.Elen.assign(n, 0); A.Degree.assign(n, 0); A.W.assign(n, 0);
  // construct A + A' lists (amd_1.c)
  std::vector<int32_t> Sp(n);
  int pfree = 0;
  for (int j = 0; j < n; j++) { A.Pe[j] = pfree; Sp[j] = pfree; pfree += A.Len[j]; }
  std::fill(Tp.begin(), Tp.end(), 0);
  for (int k = 0; k < n; k++) {
    int p;
    for (p = Ap[k]; p < Ap[k + 1];) {
      int j = Ai[p];
      if (j < k) { A.Iw[Sp[j]++] = k; A.Iw[Sp[k]++] = j; p++; }
      else if (j == k) { p++; break; }
      else break;
      int pj;
      for (pj = Tp[j]; pj < Ap[j + 1];) {
        int i = Ai[pj];
        if (i < k) { A.Iw[Sp[i]++] = j; A.Iw[Sp[j]++] = i; pj++; }
        else if (i == k) { pj++; break; }
        else break;
      }
      Tp[j] = pj;
    }
    Tp[k] = p;
  }
  for (int j = 0; j < n; j++)
    for (int pj = Tp[j]; pj < Ap[j + 1]; pj++) {
      int i = Ai[pj];
      A.Iw[Sp[i]++] = j;
      A.Iw[Sp[j]++] = i;
    }
  A.pfree = pfree;
  amd_eliminate(A, perm);
  return 0;
}

// ---------------------------------------------------------------------------
// klu_analyze (KLU/Source/klu_analyze.c order_and_analyze + analyze_worker;
// src/klu_native/analyze.rs:67-150): BTF, then AMD on each block's pattern,
// natural order for blocks of 3 or fewer.

Symbolic klu_analyze(int n, const int32_t* Ap, const int32_t* Ai) {
  Symbolic S;
  S.n = n;
  S.P.assign(n, 0);
  S.Q.assign(n, 0);
  S.R.assign(n + 1, 0);
  if (n == 0) { S.nblocks = 0; S.R.assign(1, 0); return S; }
  std::vector<int32_t> Pbtf(n), Qbtf(n), Rbtf(n + 1);
  int nmatch = 0;
  int nb = btf_order(n, Ap, Ai, Pbtf.data(), Qbtf.data(), Rbtf.data(), &nmatch);
  if (nmatch < n)
    for (int k = 0; k < n; k++) Qbtf[k] = unflip(Qbtf[k]);
  std::vector<int32_t> pinv(n);
  for (int k = 0; k < n; k++) pinv[Pbtf[k]] = k;
  std::vector<int32_t> Cp(n + 1), Ci(std::max(Ap[n], 1)), Pblk(n);
  for (int b = 0; b < nb; b++) {
    int k1 = Rbtf[b], k2 = Rbtf[b + 1], nk = k2 - k1;
    int pc = 0;
    for (int k = k1; k < k2; k++) {
      Cp[k - k1] = pc;
      int oldcol = Qbtf[k];
      for (int p = Ap[oldcol]; p < Ap[oldcol + 1]; p++) {
        int newrow = pinv[Ai[p]];
        if (newrow >= k1) Ci[pc++] = newrow - k1;
      }
    }
    Cp[nk] = pc;
    if (nk <= 3) {
      for (int k = 0; k < nk; k++) Pblk[k] = k;
    } else {
      amd_order(nk, Cp.data(), Ci.data(), Pblk.data());
    }
    for (int k = 0; k < nk; k++) {
      S.Q[k + k1] = Qbtf[Pblk[k] + k1];
      S.P[k + k1] = Pbtf[Pblk[k] + k1];
    }
  }
  S.nblocks = nb;
  S.nmatch = nmatch;
  S.R.assign(Rbtf.begin(), Rbtf.begin() + nb + 1);
  return S;
}

// ---------------------------------------------------------------------------
// First numeric factorization: Gilbert-Peierls left-looking LU per BTF
// block with threshold partial pivoting, diagonal preference and
// Eisenstat-Liu pruning (KLU/Source/klu_kernel.c KLU_kernel, klu_factor.c;
// src/klu_native/kernel.rs:341-416, factor.rs:47-131).  Unscaled, as
// KluNative runs (src/klu_native/mod.rs:44-58).

namespace {

struct BlockLU {
  // per block-local column: L rows (block-local original rows, later pivot
  // positions) and values; U rows (block-local pivot positions) and values
  std::vector<std::vector<int32_t>> li, ui;
  std::vector<std::vector<double>> lx, ux;
};

}  // namespace

int klu_factor(const Csc& A, const double* vals, const Symbolic& S, double tol, Numeric& N) {
  const int n = A.n;
  N.n = n;
  N.Pnum.assign(n, 0);
  N.Pinv.assign(n, 0);
  N.Udiag.assign(n, 0.0);
  std::vector<int32_t> psinv(n);
  for (int k = 0; k < n; k++) psinv[S.P[k]] = k;
  std::vector<std::vector<int32_t>> offrows(n);
  std::vector<std::vector<double>> offvals(n);
  std::vector<BlockLU> blocks(S.nblocks);

  for (int b = 0; b < S.nblocks; b++) {
    const int k1 = S.R[b], k2 = S.R[b + 1], nk = k2 - k1;
    BlockLU& B = blocks[b];
    B.li.assign(nk, {}); B.ui.assign(nk, {}); B.lx.assign(nk, {}); B.ux.assign(nk, {});
    std::vector<int32_t> Pb(nk), Pinvb(nk), flag(nk, EMPTY), lpend(nk, EMPTY), stack(nk),
        ap_pos(nk);
    std::vector<double> X(nk, 0.0);
    for (int k = 0; k < nk; k++) { Pb[k] = k; Pinvb[k] = flip(k); }

    for (int k = 0; k < nk; k++) {
      const int kg = k + k1, oldcol = S.Q[kg];
      std::vector<int32_t>& lik = B.li[k];
      int top = nk;
      // symbolic reach of column k (lsolve_symbolic + dfs)
      for (int p = A.p[oldcol]; p < A.p[oldcol + 1]; p++) {
        int i0 = psinv[A.i[p]] - k1;
        if (i0 < 0 || flag[i0] == k) continue;
        if (Pinvb[i0] < 0) { flag[i0] = k; lik.push_back(i0); continue; }
        int head = 0;
        stack[0] = i0;
        while (head >= 0) {
          int j = stack[head];
          int jnew = Pinvb[j];
          if (flag[j] != k) {
            flag[j] = k;
            ap_pos[head] = (lpend[jnew] == EMPTY) ? (int)B.li[jnew].size() : lpend[jnew];
          }
          const std::vector<int32_t>& Lj = B.li[jnew];
          int pos;
          for (pos = --ap_pos[head]; pos >= 0; --pos) {
            int i = Lj[pos];
            if (flag[i] == k) continue;
            if (Pinvb[i] >= 0) { ap_pos[head] = pos; stack[++head] = i; break; }
            flag[i] = k;
            lik.push_back(i);
          }
          if (pos == -1) { head--; stack[--top] = j; }
        }
      }
      // scatter column k (construct_column)
      for (int p = A.p[oldcol]; p < A.p[oldcol + 1]; p++) {
        int oldrow = A.i[p];
        int i = psinv[oldrow] - k1;
        if (i < 0) { offrows[kg].push_back(oldrow); offvals[kg].push_back(vals[p]); }
        else X[i] = vals[p];
      }
      // numeric solve with the finished columns (lsolve_numeric)
      for (int s = top; s < nk; s++) {
        int j = stack[s];
        int jnew = Pinvb[j];
        double xj = X[j];
        const std::vector<int32_t>& Lj = B.li[jnew];
        const std::vector<double>& Lxj = B.lx[jnew];
        for (size_t p = 0; p < Lj.size(); p++) X[Lj[p]] -= Lxj[p] * xj;
      }
      // partial pivoting with diagonal preference (lpivot)
      if (lik.empty()) return 1;
      int diagrow = Pb[k];
      int last_row = lik.back();
      lik.pop_back();
      std::vector<double>& lxk = B.lx[k];
      lxk.resize(lik.size());
      int pdiag = EMPTY, ppiv = EMPTY;
      double abs_pivot = EMPTY, xabs;
      for (size_t p = 0; p < lik.size(); p++) {
        int i = lik[p];
        double x = X[i];
        X[i] = 0.0;
        lxk[p] = x;
        xabs = std::fabs(x);
        if (i == diagrow) pdiag = (int)p;
        if (xabs > abs_pivot) { abs_pivot = xabs; ppiv = (int)p; }
      }
      xabs = std::fabs(X[last_row]);
      if (xabs > abs_pivot) { abs_pivot = xabs; ppiv = EMPTY; }
      if (last_row == diagrow) {
        if (xabs >= tol * abs_pivot) { abs_pivot = xabs; ppiv = EMPTY; }
      } else if (pdiag != EMPTY) {
        xabs = std::fabs(lxk[pdiag]);
        if (xabs >= tol * abs_pivot) { abs_pivot = xabs; ppiv = pdiag; }
      }
      int pivrow;
      double pivot;
      if (ppiv != EMPTY) {
        pivrow = lik[ppiv];
        pivot = lxk[ppiv];
        lik[ppiv] = last_row;
        lxk[ppiv] = X[last_row];
      } else {
        pivrow = last_row;
        pivot = X[last_row];
      }
      X[last_row] = 0.0;
      if (pivot == 0.0) return 1;
      for (double& v : lxk) v /= pivot;
      // U(:,k) from the reach, in stack order
      std::vector<int32_t>& uik = B.ui[k];
      std::vector<double>& uxk = B.ux[k];
      for (int p = top; p < nk; p++) {
        int j = stack[p];
        uik.push_back(Pinvb[j]);
        uxk.push_back(X[j]);
        X[j] = 0.0;
      }
      N.Udiag[kg] = pivot;
      if (pivrow != diagrow && Pinvb[diagrow] < 0) {
        int kbar = flip(Pinvb[pivrow]);
        Pb[kbar] = diagrow;
        Pinvb[diagrow] = flip(kbar);
      }
      Pb[k] = pivrow;
      Pinvb[pivrow] = k;
      // symmetric pruning of the columns U(:,k) touches (prune)
      for (int j : uik) {
        if (lpend[j] != EMPTY) continue;
        std::vector<int32_t>& Lj = B.li[j];
        std::vector<double>& Lxj = B.lx[j];
        if (std::find(Lj.begin(), Lj.end(), pivrow) == Lj.end()) continue;
        int phead = 0, ptail = (int)Lj.size();
        while (phead < ptail) {
          int i = Lj[phead];
          if (Pinvb[i] >= 0) phead++;
          else { ptail--; std::swap(Lj[phead], Lj[ptail]); std::swap(Lxj[phead], Lxj[ptail]); }
        }
        lpend[j] = ptail;
      }
    }
    for (int k = 0; k < nk; k++) {
      for (int32_t& r : B.li[k]) r = Pinvb[r];
      N.Pnum[k + k1] = S.P[Pb[k] + k1];
    }
  }
  for (int k = 0; k < n; k++) N.Pinv[N.Pnum[k]] = k;
  // flatten to global positions
  N.Lp.assign(n + 1, 0);
  N.Up.assign(n + 1, 0);
  N.Offp.assign(n + 1, 0);
  for (int b = 0; b < S.nblocks; b++) {
    const int k1 = S.R[b], k2 = S.R[b + 1];
    for (int k = k1; k < k2; k++) {
      const BlockLU& B = blocks[b];
      for (size_t p = 0; p < B.li[k - k1].size(); p++) {
        N.Li.push_back(B.li[k - k1][p] + k1);
        N.Lx.push_back(B.lx[k - k1][p]);
      }
      for (size_t p = 0; p < B.ui[k - k1].size(); p++) {
        N.Ui.push_back(B.ui[k - k1][p] + k1);
        N.Ux.push_back(B.ux[k - k1][p]);
      }
      N.Lp[k + 1] = (int)N.Li.size();
      N.Up[k + 1] = (int)N.Ui.size();
    }
  }
  for (int k = 0; k < n; k++) {
    for (size_t p = 0; p < offrows[k].size(); p++) {
      N.Offi.push_back(N.Pinv[offrows[k][p]]);
      N.Offx.push_back(offvals[k][p]);
    }
    N.Offp[k + 1] = (int)N.Offi.size();
  }
  return 0;
}

}  // namespace gox
