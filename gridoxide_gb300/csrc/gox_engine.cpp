// Schedule construction for the batched refactor / solve kernels and the
// host FP64 helpers used to obtain the pivot-fixing Jacobian.
#include "gox_engine.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace gox {

// power_injections (src/network.rs:680-701): S = V * conj(Y V).
void host_injections(int n, const int32_t* yp, const int32_t* yi, const double* yre,
                     const double* yim, const double* vm, const double* va, double* p,
                     double* q) {
  std::vector<double> er(n), ei(n);
  for (int k = 0; k < n; k++) { er[k] = vm[k] * std::cos(va[k]); ei[k] = vm[k] * std::sin(va[k]); }
  for (int i = 0; i < n; i++) {
    double ir = 0.0, ii = 0.0;
    for (int s = yp[i]; s < yp[i + 1]; s++) {
      int k = yi[s];
      ir += yre[s] * er[k] - yim[s] * ei[k];
      ii += yre[s] * ei[k] + yim[s] * er[k];
    }
    p[i] = er[i] * ir + ei[i] * ii;
    q[i] = ei[i] * ir - er[i] * ii;
  }
}

// JacobianPattern::fill (src/jacobian.rs:202-250).
void host_jac_fill(const JacPattern& J, const double* yre, const double* yim, const double* vm,
                   const double* va, const double* p, const double* q, double* vals) {
  for (int e = 0; e < J.nnz(); e++) {
    int i = J.bi[e], k = J.bk[e], s = J.yslot[e];
    double vi = vm[i], g = yre[s], b = yim[s], v;
    switch (J.kind[e]) {
      case K_HII: v = -q[i] - vi * vi * b; break;
      case K_NII: v = p[i] / vi + vi * g; break;
      case K_MII: v = p[i] - vi * vi * g; break;
      case K_LII: v = q[i] / vi - vi * b; break;
      default: {
        double vk = vm[k], ang = va[i] - va[k], sn = std::sin(ang), cs = std::cos(ang);
        switch (J.kind[e]) {
          case K_HIK: v = vi * vk * (g * sn - b * cs); break;
          case K_NIK: v = vi * (g * cs + b * sn); break;
          case K_MIK: v = -vi * vk * (g * cs + b * sn); break;
          default: v = vi * (g * sn - b * cs); break;
        }
      }
    }
    vals[e] = v;
  }
}

static void levels_to_lists(const std::vector<int32_t>& level, const std::vector<int32_t>& items,
                            std::vector<int32_t>& ptr, std::vector<int32_t>& out, int& nlev) {
  nlev = 0;
  for (int it : items) nlev = std::max(nlev, level[it] + 1);
  std::vector<int32_t> cnt(nlev + 1, 0);
  for (int it : items) cnt[level[it] + 1]++;
  for (int l = 0; l < nlev; l++) cnt[l + 1] += cnt[l];
  ptr.assign(cnt.begin(), cnt.end());
  out.assign(items.size(), 0);
  std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
  for (int it : items) out[fill[level[it]]++] = it;  // stable: ascending item order per level
}

void build_schedule(const JacPattern* Jp, const Csc& A, const Symbolic& S, const Numeric& N,
                    Schedule& sc) {
  const int n = A.n;
  sc = Schedule();
  sc.n_u = n;
  sc.n_bus = Jp ? Jp->n_bus : 0;
  sc.nblocks = S.nblocks;
  std::vector<int32_t> blk_of(n);
  for (int b = 0; b < S.nblocks; b++)
    for (int k = S.R[b]; k < S.R[b + 1]; k++) blk_of[k] = b;
  std::vector<int32_t> qinv(n);
  for (int k = 0; k < n; k++) qinv[S.Q[k]] = k;
  // triplet of each CSC slot (Jacobians carry no duplicate (row, col))
  std::vector<int32_t> trip_of(A.nnz(), -1);
  for (int e = 0; e < (int)A.slot_of.size(); e++) {
    if (Jp && trip_of[A.slot_of[e]] != -1) throw std::runtime_error("duplicate Jacobian entry");
    if (trip_of[A.slot_of[e]] == -1) trip_of[A.slot_of[e]] = e;
  }

  // ---- per-column layout: [U (topological order) | diag | L]
  sc.c_base.assign(n, 0); sc.c_ulen.assign(n, 0); sc.c_llen.assign(n, 0);
  int slot = 0;
  for (int k = 0; k < n; k++) {
    sc.c_ulen[k] = N.Up[k + 1] - N.Up[k];
    sc.c_llen[k] = N.Lp[k + 1] - N.Lp[k];
    sc.c_base[k] = slot;
    slot += sc.c_ulen[k] + 1 + sc.c_llen[k];
    sc.max_collen = std::max(sc.max_collen, sc.c_ulen[k] + 1 + sc.c_llen[k]);
  }
  sc.n_slots = slot;
  auto lslot = [&](int j, int t) { return sc.c_base[j] + sc.c_ulen[j] + 1 + t; };
  auto uslot = [&](int j, int p) { return sc.c_base[j] + p; };

  // ---- A entries (scatter of A(:, Q[k]) in CSC order), ops
  std::vector<int32_t> pos_of(n, -1);
  sc.c_abeg.assign(n + 1, 0);
  sc.c_obeg.assign(n + 1, 0);
  sc.op_ptr.assign(n + 1, 0);
  int noff = 0;
  for (int k = 0; k < n; k++) {
    const int ulen = sc.c_ulen[k], llen = sc.c_llen[k];
    for (int p = 0; p < ulen; p++) pos_of[N.Ui[N.Up[k] + p]] = p;
    pos_of[k] = ulen;
    for (int t = 0; t < llen; t++) pos_of[N.Li[N.Lp[k] + t]] = ulen + 1 + t;
    const int k1 = S.R[blk_of[k]];
    const int oldcol = S.Q[k];
    sc.c_abeg[k] = (int)sc.a_dst.size();
    sc.c_obeg[k] = noff;
    for (int p = A.p[oldcol]; p < A.p[oldcol + 1]; p++) {
      int newrow = N.Pinv[A.i[p]];
      int e = trip_of[p];
      sc.a_kind.push_back(Jp ? Jp->kind[e] : 0);
      sc.a_bi.push_back(Jp ? Jp->bi[e] : 0);
      sc.a_bk.push_back(Jp ? Jp->bk[e] : 0);
      sc.a_yslot.push_back(Jp ? Jp->yslot[e] : 0);
      if (newrow < k1) {
        sc.a_dst.push_back(-(noff + 1));
        noff++;
      } else {
        int d = pos_of[newrow];
        if (d < 0) throw std::runtime_error("A entry outside the factor pattern");
        sc.a_dst.push_back(d);
      }
    }
    for (int p = 0; p < ulen; p++) {
      int j = N.Ui[N.Up[k] + p];
      for (int t = 0; t < sc.c_llen[j]; t++) {
        int row = N.Li[N.Lp[j] + t];
        int d = pos_of[row];
        if (d < 0 || d <= p) throw std::runtime_error("update outside the column pattern");
        sc.op_slot.push_back(lslot(j, t));
        sc.op_pos.push_back((uint32_t)d | ((uint32_t)p << 16));
      }
      sc.flops_refactor += 2.0 * sc.c_llen[j];
    }
    sc.flops_refactor += llen;
    sc.op_ptr[k + 1] = (int)sc.op_slot.size();
    for (int p = 0; p < ulen; p++) pos_of[N.Ui[N.Up[k] + p]] = -1;
    pos_of[k] = -1;
    for (int t = 0; t < llen; t++) pos_of[N.Li[N.Lp[k] + t]] = -1;
  }
  sc.c_abeg[n] = (int)sc.a_dst.size();
  sc.c_obeg[n] = noff;
  sc.n_a = (int)sc.a_dst.size();
  sc.n_off = noff;
  if (sc.max_collen >= 65536) throw std::runtime_error("column too long for 16-bit stage positions");

  // ---- refactor levels: column k waits for every j in U(:, k)
  std::vector<int32_t> level(n, 0), cols(n);
  for (int k = 0; k < n; k++) {
    int lv = 0;
    for (int p = N.Up[k]; p < N.Up[k + 1]; p++) lv = std::max(lv, level[N.Ui[p]] + 1);
    level[k] = lv;
    cols[k] = k;
  }
  levels_to_lists(level, cols, sc.lev_ptr, sc.lev_cols, sc.n_levels);

  // ---- row-oriented solve lists
  std::vector<std::vector<std::pair<int32_t, int32_t>>> lrow(n), urow(n), orow(n);
  for (int j = 0; j < n; j++) {
    for (int t = 0; t < sc.c_llen[j]; t++) lrow[N.Li[N.Lp[j] + t]].push_back({lslot(j, t), j});
    for (int p = 0; p < sc.c_ulen[j]; p++) urow[N.Ui[N.Up[j] + p]].push_back({uslot(j, p), j});
  }
  for (int j = 0; j < n; j++) {
    for (int a = sc.c_abeg[j]; a < sc.c_abeg[j + 1]; a++) {
      if (sc.a_dst[a] >= 0) continue;
      int off = -sc.a_dst[a] - 1;
      // row of this off entry in pivot order
      int p = A.p[S.Q[j]] + (a - sc.c_abeg[j]);
      int row = N.Pinv[A.i[p]];
      orow[row].push_back({-(off + 1), j});
    }
  }
  sc.fw_ptr.assign(n + 1, 0);
  sc.bw_ptr.assign(n + 1, 0);
  sc.diag_slot.assign(n, 0);
  for (int k = 0; k < n; k++) {
    for (auto& t : orow[k]) { sc.fw_slot.push_back(t.first); sc.fw_col.push_back(t.second); }
    for (auto& t : lrow[k]) { sc.fw_slot.push_back(t.first); sc.fw_col.push_back(t.second); }
    sc.fw_ptr[k + 1] = (int)sc.fw_slot.size();
    for (auto& t : urow[k]) { sc.bw_slot.push_back(t.first); sc.bw_col.push_back(t.second); }
    sc.bw_ptr[k + 1] = (int)sc.bw_slot.size();
    sc.diag_slot[k] = sc.c_base[k] + sc.c_ulen[k];
    sc.flops_solve += 2.0 * (lrow[k].size() + urow[k].size() + orow[k].size()) + 1;
  }
  // phases: blocks in reverse order; forward levels then backward levels
  sc.ph_ptr.assign(1, 0);
  std::vector<int32_t> fl(n, 0), bl(n, 0);
  for (int b = S.nblocks - 1; b >= 0; b--) {
    const int k1 = S.R[b], k2 = S.R[b + 1];
    std::vector<int32_t> rows;
    for (int k = k1; k < k2; k++) {
      int lv = 0;
      for (auto& t : lrow[k]) lv = std::max(lv, fl[t.second] + 1);
      fl[k] = lv;
      rows.push_back(k);
    }
    for (int k = k2 - 1; k >= k1; k--) {
      int lv = 0;
      for (auto& t : urow[k]) lv = std::max(lv, bl[t.second] + 1);
      bl[k] = lv;
    }
    std::vector<int32_t> ptr, out;
    int nl;
    levels_to_lists(fl, rows, ptr, out, nl);
    for (int l = 0; l < nl; l++) {
      for (int q = ptr[l]; q < ptr[l + 1]; q++) sc.ph_rows.push_back(out[q]);
      sc.ph_ptr.push_back((int)sc.ph_rows.size());
      sc.ph_kind.push_back(0);
    }
    levels_to_lists(bl, rows, ptr, out, nl);
    for (int l = 0; l < nl; l++) {
      for (int q = ptr[l]; q < ptr[l + 1]; q++) sc.ph_rows.push_back(out[q]);
      sc.ph_ptr.push_back((int)sc.ph_rows.size());
      sc.ph_kind.push_back(1);
    }
  }
  sc.n_phases = (int)sc.ph_kind.size();

  // ---- bus <-> permuted rhs rows / solution entries
  if (!Jp) return;
  const JacPattern& J = *Jp;
  const int nb = J.n_bus;
  sc.bus_rowP.assign(nb, -1); sc.bus_rowQ.assign(nb, -1);
  sc.bus_colA.assign(nb, -1); sc.bus_colV.assign(nb, -1);
  for (int i = 0; i < nb; i++) {
    if (J.ns_pos[i] >= 0) {
      int u = J.ns_pos[i];
      sc.bus_rowP[i] = N.Pinv[u];
      sc.bus_colA[i] = qinv[u];
    }
    if (J.pq_pos[i] >= 0) {
      int u = J.n_ang + J.pq_pos[i];
      sc.bus_rowQ[i] = N.Pinv[u];
      sc.bus_colV[i] = qinv[u];
    }
  }
}

}  // namespace gox
