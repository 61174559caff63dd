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
  if (sc.max_collen * 32 >= 65536)
    throw std::runtime_error("column too long for 16-bit stage offsets");
  auto lslot = [&](int j, int t) { return sc.c_base[j] + sc.c_ulen[j] + 1 + t; };
  auto uslot = [&](int j, int p) { return sc.c_base[j] + p; };

  // ---- off-diagonal (BTF) entries, numbered column by column in CSC order
  //      (the order KLU's construct_column emits them)
  std::vector<int32_t> off_of_p(A.nnz(), -1);
  int noff = 0;
  for (int k = 0; k < n; k++) {
    const int k1 = S.R[blk_of[k]];
    for (int p = A.p[S.Q[k]]; p < A.p[S.Q[k] + 1]; p++)
      if (N.Pinv[A.i[p]] < k1) off_of_p[p] = noff++;
  }
  sc.n_off = noff;
  sc.fuse_fwd = (noff == 0);

  // ---- row lists for the substitutions
  std::vector<std::vector<std::pair<int32_t, int32_t>>> lrow(n), urow(n), orow(n);
  for (int j = 0; j < n; j++) {
    for (int t = 0; t < sc.c_llen[j]; t++) lrow[N.Li[N.Lp[j] + t]].push_back({lslot(j, t), j});
    for (int p = 0; p < sc.c_ulen[j]; p++) urow[N.Ui[N.Up[j] + p]].push_back({uslot(j, p), j});
    for (int p = A.p[S.Q[j]]; p < A.p[S.Q[j] + 1]; p++)
      if (off_of_p[p] >= 0) orow[N.Pinv[A.i[p]]].push_back({-(off_of_p[p] + 1), j});
  }

  // ---- refactor levels: column k waits for every j in U(:, k) (and, when
  //      the forward substitution is fused, for every j with L(k, j) != 0)
  std::vector<int32_t> level(n, 0), cols(n);
  for (int k = 0; k < n; k++) {
    int lv = 0;
    for (int p = N.Up[k]; p < N.Up[k + 1]; p++) lv = std::max(lv, level[N.Ui[p]] + 1);
    if (sc.fuse_fwd)
      for (auto& t : lrow[k]) lv = std::max(lv, level[t.second] + 1);
    level[k] = lv;
    cols[k] = k;
  }
  levels_to_lists(level, cols, sc.lev_ptr, sc.lev_cols, sc.n_levels);

  // ---- A entries (scatter of A(:, Q[k]) in CSC order), emitted in the
  //      order the refactor consumes columns; ops per column
  std::vector<int32_t> pos_of(n, -1);
  sc.c_abeg.assign(n, 0);
  sc.c_aend.assign(n, 0);
  for (int q = 0; q < n; q++) {
    const int k = sc.lev_cols[q];
    const int ulen = sc.c_ulen[k], llen = sc.c_llen[k];
    for (int p = 0; p < ulen; p++) pos_of[N.Ui[N.Up[k] + p]] = p;
    pos_of[k] = ulen;
    for (int t = 0; t < llen; t++) pos_of[N.Li[N.Lp[k] + t]] = ulen + 1 + t;
    sc.c_abeg[k] = (int)sc.a_dst.size();
    for (int p = A.p[S.Q[k]]; p < A.p[S.Q[k] + 1]; p++) {
      int e = trip_of[p];
      sc.a_kind.push_back(Jp ? Jp->kind[e] : 0);
      sc.a_bi.push_back(Jp ? Jp->bi[e] : 0);
      sc.a_bk.push_back(Jp ? Jp->bk[e] : 0);
      sc.a_yslot.push_back(Jp ? Jp->yslot[e] : 0);
      sc.a_csc.push_back(p);
      if (off_of_p[p] >= 0) {
        sc.a_dst.push_back(-(off_of_p[p] + 1));
      } else {
        int d = pos_of[N.Pinv[A.i[p]]];
        if (d < 0) throw std::runtime_error("A entry outside the factor pattern");
        sc.a_dst.push_back(d);
      }
    }
    sc.c_aend[k] = (int)sc.a_dst.size();
    for (int t = 0; t < llen; t++) pos_of[N.Li[N.Lp[k] + t]] = -1;
    pos_of[k] = -1;
    for (int p = 0; p < ulen; p++) pos_of[N.Ui[N.Up[k] + p]] = -1;
  }
  sc.n_a = (int)sc.a_dst.size();
  // ---- update ops of each column, in left-looking order (U(:,k) in
  //      topological order, each j's L(:,j) rows in stored order), then
  //      regrouped into hazard-free batches by ASAP levels:
  //        RAW  an op reading stage entry u waits for the last writer of u
  //        WAW  an op writing d waits for the last writer of d (so every
  //             entry receives its contributions in the original order and
  //             the rounding is that of the sequential loop)
  //        WAR  an op writing d may share a batch with an earlier reader of
  //             d (batches load before they store) but not precede it
  sc.op_ptr.assign(n + 1, 0);
  sc.bt_ptr.assign(n + 1, 0);
  sc.col_level = level;
  sc.cu_ptr.assign(n + 1, 0);
  sc.cu_dptr.assign(1, 0);
  std::vector<int32_t> lastw(sc.max_collen + 1, -1), maxr(sc.max_collen + 1, -1);
  struct Op { int32_t dst, up, slot, lev; };
  std::vector<Op> ops;
  for (int k = 0; k < n; k++) {
    const int ulen = sc.c_ulen[k], llen = sc.c_llen[k];
    const int len = ulen + 1 + llen;
    for (int p = 0; p < ulen; p++) pos_of[N.Ui[N.Up[k] + p]] = p;
    pos_of[k] = ulen;
    for (int t = 0; t < llen; t++) pos_of[N.Li[N.Lp[k] + t]] = ulen + 1 + t;
    ops.clear();
    for (int p = 0; p < ulen; p++) {
      int j = N.Ui[N.Up[k] + p];
      for (int t = 0; t < sc.c_llen[j]; t++) {
        int d = pos_of[N.Li[N.Lp[j] + t]];
        if (d < 0 || d <= p) throw std::runtime_error("update outside the column pattern");
        ops.push_back({d, p, lslot(j, t), 0});
        sc.cu_dst.push_back(d);
      }
      sc.cu_j.push_back(j);
      sc.cu_dptr.push_back((int32_t)sc.cu_dst.size());
      sc.flops_refactor += 2.0 * sc.c_llen[j];
    }
    sc.flops_refactor += llen;
    std::fill(lastw.begin(), lastw.begin() + len, -1);
    std::fill(maxr.begin(), maxr.begin() + len, -1);
    int nlev = 0;
    for (auto& o : ops) {
      int lv = 0;
      if (lastw[o.up] >= 0) lv = std::max(lv, lastw[o.up] + 1);
      if (lastw[o.dst] >= 0) lv = std::max(lv, lastw[o.dst] + 1);
      lv = std::max(lv, maxr[o.dst]);
      o.lev = lv;
      lastw[o.dst] = lv;
      maxr[o.up] = std::max(maxr[o.up], lv);
      nlev = std::max(nlev, lv + 1);
    }
    std::vector<std::vector<int32_t>> bylev(nlev);
    for (int i = 0; i < (int)ops.size(); i++) bylev[ops[i].lev].push_back(i);
    for (auto& L : bylev) {
      for (size_t c = 0; c < L.size(); c += kMaxBatch) {
        size_t e = std::min(L.size(), c + kMaxBatch);
        for (size_t q = c; q < e; q++) {
          const Op& o = ops[L[q]];
          sc.op_slot.push_back(o.slot);
          sc.op_pos.push_back((uint32_t)o.dst | ((uint32_t)o.up << 16));
        }
        sc.bt_cnt.push_back((uint8_t)(e - c));
      }
    }
    sc.op_ptr[k + 1] = (int)sc.op_slot.size();
    sc.cu_ptr[k + 1] = (int)sc.cu_j.size();
    sc.bt_ptr[k + 1] = (int)sc.bt_cnt.size();
    sc.max_ops = std::max(sc.max_ops, (int)ops.size());
    sc.max_batches = std::max(sc.max_batches, sc.bt_ptr[k + 1] - sc.bt_ptr[k]);
    for (int t = 0; t < llen; t++) pos_of[N.Li[N.Lp[k] + t]] = -1;
    pos_of[k] = -1;
    for (int p = 0; p < ulen; p++) pos_of[N.Ui[N.Up[k] + p]] = -1;
  }

  // ---- substitution term lists
  sc.fw_ptr.assign(n + 1, 0);
  sc.bw_ptr.assign(n + 1, 0);
  sc.diag_slot.assign(n, 0);
  for (int k = 0; k < n; k++) {
    for (auto& t : orow[k]) { sc.fw_slot.push_back(t.first); sc.fw_col.push_back(t.second); }
    for (auto& t : lrow[k]) { sc.fw_slot.push_back(t.first); sc.fw_col.push_back(t.second); }
    sc.fw_ptr[k + 1] = (int)sc.fw_slot.size();
    sc.max_fw = std::max(sc.max_fw, sc.fw_ptr[k + 1] - sc.fw_ptr[k]);
    for (auto& t : urow[k]) { sc.bw_slot.push_back(t.first); sc.bw_col.push_back(t.second); }
    sc.bw_ptr[k + 1] = (int)sc.bw_slot.size();
    sc.diag_slot[k] = sc.c_base[k] + sc.c_ulen[k];
    sc.flops_solve += 2.0 * (lrow[k].size() + urow[k].size() + orow[k].size()) + 1;
  }
  // phases: blocks in reverse order; forward levels (unless fused into the
  // refactor) then backward levels
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
    if (!sc.fuse_fwd) {
      levels_to_lists(fl, rows, ptr, out, nl);
      for (int l = 0; l < nl; l++) {
        for (int q = ptr[l]; q < ptr[l + 1]; q++) sc.ph_rows.push_back(out[q]);
        sc.ph_ptr.push_back((int)sc.ph_rows.size());
        sc.ph_kind.push_back(0);
      }
    }
    levels_to_lists(bl, rows, ptr, out, nl);
    for (int l = 0; l < nl; l++) {
      for (int q = ptr[l]; q < ptr[l + 1]; q++) sc.ph_rows.push_back(out[q]);
      sc.ph_ptr.push_back((int)sc.ph_rows.size());
      sc.ph_kind.push_back(1);
    }
  }
  if (sc.fuse_fwd) {
    // without off-diagonal blocks the blocks are independent: merge their
    // backward levels so one phase spans every block
    std::vector<int32_t> ptr, out, all(n);
    int nl;
    for (int k = 0; k < n; k++) all[k] = k;
    levels_to_lists(bl, all, ptr, out, nl);
    sc.ph_ptr.assign(1, 0);
    sc.ph_rows.clear();
    sc.ph_kind.clear();
    for (int l = 0; l < nl; l++) {
      for (int q = ptr[l]; q < ptr[l + 1]; q++) sc.ph_rows.push_back(out[q]);
      sc.ph_ptr.push_back((int)sc.ph_rows.size());
      sc.ph_kind.push_back(1);
    }
  }
  sc.n_phases = (int)sc.ph_kind.size();

  // ---- per-column packets in consumption order
  sc.pk_off.assign(n + 1, 0);
  for (int q = 0; q < n; q++) {
    const int k = sc.lev_cols[q];
    sc.pk_off[q] = (int)sc.pk.size();
    const int nA = sc.c_aend[k] - sc.c_abeg[k];
    const int ob = sc.op_ptr[k], nops = sc.op_ptr[k + 1] - ob;
    const int bb = sc.bt_ptr[k], nbt = sc.bt_ptr[k + 1] - bb;
    const int fb = sc.fw_ptr[k], nfw = sc.fuse_fwd ? sc.fw_ptr[k + 1] - fb : 0;
    int32_t hdr[12] = {k, sc.c_base[k], sc.c_ulen[k], sc.c_llen[k], nA, nops, nbt, nfw,
                       sc.c_abeg[k], ob, 0, 0};
    sc.pk.insert(sc.pk.end(), hdr, hdr + 12);
    for (int a = sc.c_abeg[k]; a < sc.c_aend[k]; a++) sc.pk.push_back(sc.a_dst[a]);
    for (int t = 0; t < nfw; t++) { sc.pk.push_back(sc.fw_slot[fb + t]); sc.pk.push_back(sc.fw_col[fb + t]); }
    for (int t = 0; t < nbt; t += 4) {
      uint32_t w = 0;
      for (int c = 0; c < 4 && t + c < nbt; c++) w |= (uint32_t)sc.bt_cnt[bb + t + c] << (8 * c);
      sc.pk.push_back((int32_t)w);
    }
    sc.max_head = std::max(sc.max_head, (int)sc.pk.size() - sc.pk_off[q]);
    for (int t = 0; t < nops; t++) {
      const uint32_t ps = sc.op_pos[ob + t];
      sc.pk.push_back(sc.op_slot[ob + t] * 32);
      sc.pk.push_back((int32_t)(((ps & 0xffffu) * 32u) | (((ps >> 16) * 32u) << 16)));
    }
    while (sc.pk.size() % 4) sc.pk.push_back(0);
    sc.max_pk = std::max(sc.max_pk, (int)sc.pk.size() - sc.pk_off[q]);
  }
  sc.pk_off[n] = (int)sc.pk.size();
  // ---- fill recipe in LU layout
  sc.slot_a.assign(sc.n_slots, -1);
  sc.off_a.assign(sc.n_off, -1);
  for (int k = 0; k < n; k++)
    for (int a = sc.c_abeg[k]; a < sc.c_aend[k]; a++) {
      if (sc.a_dst[a] >= 0) sc.slot_a[sc.c_base[k] + sc.a_dst[a]] = a;
      else sc.off_a[-sc.a_dst[a] - 1] = a;
    }

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
