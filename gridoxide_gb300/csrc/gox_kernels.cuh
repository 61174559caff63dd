// CUDA kernels of the batched Newton-Raphson path (sm_103a).
//
// Lane l of the warps of CTA g works on scenario 32*g + l; all lanes run
// the same instruction stream on their own scenario's values, so every
// global access is one coalesced transaction (see gox_engine.hpp for the
// layout) and every schedule read is a warp-uniform broadcast.
//
//   k_mismatch  K1 (+K5): apply the previous Newton step, V = |V|e^{j theta},
//               S = V conj(Y V), mismatch F, max|F|, convergence.  FP64.
//   k_fill      K2: Jacobian values in the refactor's consumption order,
//               trig-free rectangular form.  FP64 or FP32 output.
//   k_refactor  K3: level-synchronous left-looking refactorization with the
//               static pivot order; each warp stages its column in shared
//               memory.  FP64 or FP32.
//   k_solve     K4: row-oriented forward/backward substitution, BTF blocks
//               in reverse order.  FP64 or FP32.
// None of them waits on another CTA: only __syncthreads inside a CTA.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gox {

enum : int { ST_RUNNING = -1, ST_CONVERGED = 0, ST_MAXITER = 1, ST_SINGULAR = 2, ST_UNUSED = 3 };

struct SchedDev {
  int n_bus, n_u, n_a, n_slots, n_off, n_levels, n_phases, nnz_y;
  const int32_t *yp, *yi;
  const double *yre, *yim;
  const int32_t *bus_rowP, *bus_rowQ, *bus_colA, *bus_colV;
  const int32_t *a_kind, *a_bi, *a_bk, *a_yslot, *a_dst;
  const int32_t *lev_ptr, *lev_cols, *c_base, *c_ulen, *c_llen, *c_abeg, *op_ptr, *op_slot;
  const uint32_t* op_pos;
  const int32_t *ph_ptr, *ph_rows, *ph_kind, *fw_ptr, *fw_slot, *fw_col, *bw_ptr, *bw_slot,
      *bw_col, *diag_slot;
};

struct BatchDev {
  int G;          // groups of 32 scenarios
  int max_iter;
  double tol;
  // FP64 state [G][n_bus][32]
  double *vm, *va, *e, *f, *psp, *qsp;
  // typed working arrays (T = float or double)
  void *eT, *fT, *ivT, *pT, *qT;  // [G][n_bus][32]
  void *jbuf;                      // [G][n_a][32]
  void *lu;                        // [G][n_slots][32]
  void *off;                       // [G][n_off][32]
  void *rhs, *sol;                 // [G][n_u][32]
  // per scenario [G*32]
  int32_t *status, *iters, *sing, *piv_flag;
  double *maxmis;
  double *hist;                    // [G*32][max_iter] or null
  int32_t *gact;                   // [G] group has a running lane
  int32_t *nactive;                // [1] running groups after the last mismatch
  // optional per-scenario outage: 4 Y slots + deltas, and the branch buses
  const int32_t *o_slot, *o_bf, *o_bt;
  const double *o_dre, *o_dim;
  float piv_tol;                   // pivot-ratio threshold (mixed path)
};

__device__ __forceinline__ size_t gidx(int g, int n, int e, int lane) {
  return ((size_t)g * (size_t)n + (size_t)e) * 32u + (size_t)lane;
}

// ---------------------------------------------------------------------------
// K1 (+K5): update, injections, mismatch, convergence.  One CTA per group.
// mode 0: iteration `it` (update if it > 0, then mismatch)
// mode 1: final update after the last allowed iteration (no mismatch)
template <typename T, bool OUTAGE>
__global__ void __launch_bounds__(256) k_mismatch(SchedDev S, BatchDev D, int it, int mode) {
  const int g = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int s = g * 32 + lane;
  const int N = S.n_bus;
  __shared__ double red[32][33];
  __shared__ int run_sh[32];

  int st = D.status[s];
  bool running = (st == ST_RUNNING);
  bool do_update = running && (it > 0 || mode == 1);
  if (running && (it > 0 || mode == 1) && D.sing[s]) {
    // the previous refactor/solve failed: Singular, voltages untouched
    running = false;
    do_update = false;
    if (warp == 0) D.status[s] = ST_SINGULAR;
  }
  const T* sol = (const T*)D.sol;
  // ---- pass A: apply dx and form V = |V| e^{j theta}
  for (int i = warp; i < N; i += nw) {
    size_t x = gidx(g, N, i, lane);
    double vm = D.vm[x], va = D.va[x];
    if (do_update) {
      int ca = S.bus_colA[i], cv = S.bus_colV[i];
      if (ca >= 0) va += (double)sol[gidx(g, S.n_u, ca, lane)];
      if (cv >= 0) vm += (double)sol[gidx(g, S.n_u, cv, lane)];
      D.vm[x] = vm;
      D.va[x] = va;
    }
    if (mode == 0) {
      double sn, cs;
      sincos(va, &sn, &cs);
      D.e[x] = vm * cs;
      D.f[x] = vm * sn;
    }
  }
  if (mode == 1) {
    if (running && warp == 0) {
      D.status[s] = ST_MAXITER;
    }
    return;
  }
  __syncthreads();
  // ---- pass B: I = Y V, S = V conj(I), mismatch
  T* rhs = (T*)D.rhs;
  T* eT = (T*)D.eT; T* fT = (T*)D.fT; T* ivT = (T*)D.ivT; T* pT = (T*)D.pT; T* qT = (T*)D.qT;
  int obf = -1, obt = -1;
  double o_ff_r = 0, o_ff_i = 0, o_ft_r = 0, o_ft_i = 0, o_tf_r = 0, o_tf_i = 0, o_tt_r = 0, o_tt_i = 0;
  if (OUTAGE) {
    obf = D.o_bf[s];
    obt = D.o_bt[s];
    if (obf >= 0) {
      o_ff_r = D.o_dre[4 * s + 0]; o_ff_i = D.o_dim[4 * s + 0];
      o_ft_r = D.o_dre[4 * s + 1]; o_ft_i = D.o_dim[4 * s + 1];
      o_tf_r = D.o_dre[4 * s + 2]; o_tf_i = D.o_dim[4 * s + 2];
      o_tt_r = D.o_dre[4 * s + 3]; o_tt_i = D.o_dim[4 * s + 3];
    }
  }
  double mx = 0.0;
  for (int i = warp; i < N; i += nw) {
    double ir = 0.0, ii = 0.0;
    const int pb = S.yp[i], pe = S.yp[i + 1];
    for (int p = pb; p < pe; p++) {
      const int k = __ldg(S.yi + p);
      const double gr = __ldg(S.yre + p), gi = __ldg(S.yim + p);
      size_t xk = gidx(g, N, k, lane);
      double ek = D.e[xk], fk = D.f[xk];
      ir += gr * ek - gi * fk;
      ii += gr * fk + gi * ek;
    }
    size_t x = gidx(g, N, i, lane);
    double ei = D.e[x], fi = D.f[x];
    if (OUTAGE) {
      if (i == obf || i == obt) {
        size_t xf = gidx(g, N, obf, lane), xt = gidx(g, N, obt, lane);
        double ef = D.e[xf], ff = D.f[xf], et = D.e[xt], ft = D.f[xt];
        if (i == obf) {
          ir += o_ff_r * ef - o_ff_i * ff + o_ft_r * et - o_ft_i * ft;
          ii += o_ff_r * ff + o_ff_i * ef + o_ft_r * ft + o_ft_i * et;
        } else {
          ir += o_tf_r * ef - o_tf_i * ff + o_tt_r * et - o_tt_i * ft;
          ii += o_tf_r * ff + o_tf_i * ef + o_tt_r * ft + o_tt_i * et;
        }
      }
    }
    double pc = ei * ir + fi * ii;
    double qc = fi * ir - ei * ii;
    int rp = S.bus_rowP[i], rq = S.bus_rowQ[i];
    if (running) {
      if (rp >= 0) {
        double F = D.psp[x] - pc;
        mx = fmax(mx, fabs(F));
        rhs[gidx(g, S.n_u, rp, lane)] = (T)F;
      }
      if (rq >= 0) {
        double F = D.qsp[x] - qc;
        mx = fmax(mx, fabs(F));
        rhs[gidx(g, S.n_u, rq, lane)] = (T)F;
      }
    }
    double vm = D.vm[x];
    eT[x] = (T)ei;
    fT[x] = (T)fi;
    ivT[x] = (T)(1.0 / vm);
    pT[x] = (T)pc;
    qT[x] = (T)qc;
  }
  red[warp][lane] = mx;
  __syncthreads();
  if (warp == 0) {
    double m = 0.0;
    for (int w = 0; w < nw; w++) m = fmax(m, red[w][lane]);
    if (running) {
      D.maxmis[s] = m;
      if (D.hist) D.hist[(size_t)s * D.max_iter + it] = m;
      D.iters[s] = it + 1;
      D.sing[s] = (D.sing[s] == 2) ? 2 : 0;  // 2: the scenario's own first factorization failed
      if (m < D.tol) {
        D.status[s] = ST_CONVERGED;
        running = false;
      }
    }
    unsigned any = __ballot_sync(0xffffffffu, running);
    if (lane == 0) {
      D.gact[g] = any ? 1 : 0;
      if (any) atomicAdd(D.nactive, 1);
    }
  }
  (void)run_sh;
}

// ---------------------------------------------------------------------------
// K2: Jacobian fill (src/jacobian.rs:202-250 formulas in rectangular form:
// V_i V_k cos(th_i - th_k) = e_i e_k + f_i f_k, V_i V_k sin(...) = f_i e_k - e_i f_k).
// grid (chunks, G); each warp fills a contiguous run of entries.
template <typename T, bool OUTAGE>
__global__ void __launch_bounds__(256) k_fill(SchedDev S, BatchDev D, int per_warp) {
  const int g = blockIdx.y;
  if (!D.gact[g]) return;
  const int lane = threadIdx.x & 31;
  const int wglob = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int a0 = wglob * per_warp;
  if (a0 >= S.n_a) return;
  const int a1 = min(S.n_a, a0 + per_warp);
  const int N = S.n_bus;
  const int s = g * 32 + lane;
  const T* eT = (const T*)D.eT; const T* fT = (const T*)D.fT; const T* ivT = (const T*)D.ivT;
  const T* pT = (const T*)D.pT; const T* qT = (const T*)D.qT;
  T* J = (T*)D.jbuf;
  int os0 = -1, os1 = -1, os2 = -1, os3 = -1;
  if (OUTAGE && D.o_bf[s] >= 0) {
    os0 = D.o_slot[4 * s]; os1 = D.o_slot[4 * s + 1]; os2 = D.o_slot[4 * s + 2]; os3 = D.o_slot[4 * s + 3];
  }
  for (int a = a0; a < a1; a++) {
    const int kind = __ldg(S.a_kind + a), i = __ldg(S.a_bi + a), k = __ldg(S.a_bk + a);
    const int ys = __ldg(S.a_yslot + a);
    double gd = __ldg(S.yre + ys), bd = __ldg(S.yim + ys);
    if (OUTAGE) {
      int c = (ys == os0) ? 0 : (ys == os1) ? 1 : (ys == os2) ? 2 : (ys == os3) ? 3 : -1;
      if (c >= 0) { gd += D.o_dre[4 * s + c]; bd += D.o_dim[4 * s + c]; }
    }
    const T G = (T)gd, B = (T)bd;
    const size_t xi = gidx(g, N, i, lane);
    T v;
    if (kind == 0 || kind == 1 || kind == 4 || kind == 5) {
      const T ei = eT[xi], fi = fT[xi], iv = ivT[xi];
      const T vi2 = ei * ei + fi * fi;
      const T vi = vi2 * iv;  // |V_i|^2 / |V_i|
      const T P = pT[xi], Q = qT[xi];
      switch (kind) {
        case 0: v = -Q - vi2 * B; break;            // H_ii
        case 1: v = P * iv + vi * G; break;         // N_ii
        case 4: v = P - vi2 * G; break;             // M_ii
        default: v = Q * iv - vi * B; break;        // L_ii
      }
    } else {
      const size_t xk = gidx(g, N, k, lane);
      const T ei = eT[xi], fi = fT[xi], ek = eT[xk], fk = fT[xk];
      const T c = ei * ek + fi * fk;   // V_i V_k cos
      const T sn = fi * ek - ei * fk;  // V_i V_k sin
      switch (kind) {
        case 2: v = G * sn - B * c; break;                 // H_ik
        case 3: v = (G * c + B * sn) * ivT[xk]; break;     // N_ik
        case 6: v = -(G * c + B * sn); break;              // M_ik
        default: v = (G * sn - B * c) * ivT[xk]; break;    // L_ik
      }
    }
    J[gidx(g, S.n_a, a, lane)] = v;
  }
}

// ---------------------------------------------------------------------------
// K3: refactor.  One CTA per group; columns of a dependency level are dealt
// to warps; __syncthreads between levels.  Stage layout per column:
// [U entries (topological order) | diagonal | L entries].
template <typename T>
__global__ void __launch_bounds__(256) k_refactor(SchedDev S, BatchDev D, int cap) {
  const int g = blockIdx.x;
  if (!D.gact[g]) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T* stage_w = reinterpret_cast<T*>(smem_raw) + (size_t)warp * cap * 32;
  const int s = g * 32 + lane;
  T* LU = (T*)D.lu;
  T* OFF = (T*)D.off;
  const T* J = (const T*)D.jbuf;
  const size_t luG = (size_t)g * S.n_slots * 32u;
  bool bad = false, tiny = false;
  const float ptol = D.piv_tol;

  for (int lv = 0; lv < S.n_levels; lv++) {
    const int q0 = __ldg(S.lev_ptr + lv), q1 = __ldg(S.lev_ptr + lv + 1);
    for (int q = q0 + warp; q < q1; q += nw) {
      const int k = __ldg(S.lev_cols + q);
      const int base = __ldg(S.c_base + k), ulen = __ldg(S.c_ulen + k), llen = __ldg(S.c_llen + k);
      const int len = ulen + 1 + llen;
      T* st = (len <= cap) ? stage_w : (LU + luG + (size_t)base * 32u);
      for (int p = 0; p < len; p++) st[p * 32 + lane] = (T)0;
      const int ab = __ldg(S.c_abeg + k), ae = __ldg(S.c_abeg + k + 1);
      for (int a = ab; a < ae; a++) {
        const int d = __ldg(S.a_dst + a);
        const T v = J[gidx(g, S.n_a, a, lane)];
        if (d >= 0) st[d * 32 + lane] = v;
        else OFF[gidx(g, S.n_off, -d - 1, lane)] = v;
      }
      const int ob = __ldg(S.op_ptr + k), oe = __ldg(S.op_ptr + k + 1);
      int o = ob;
      for (; o + 8 <= oe; o += 8) {
        T lv8[8];
        uint32_t ps[8];
#pragma unroll
        for (int t = 0; t < 8; t++) {
          ps[t] = __ldg(S.op_pos + o + t);
          lv8[t] = LU[luG + (size_t)__ldg(S.op_slot + o + t) * 32u + lane];
        }
#pragma unroll
        for (int t = 0; t < 8; t++) {
          const int dst = ps[t] & 0xffff, up = ps[t] >> 16;
          st[dst * 32 + lane] -= lv8[t] * st[up * 32 + lane];
        }
      }
      for (; o < oe; o++) {
        const uint32_t ps = __ldg(S.op_pos + o);
        const T lvv = LU[luG + (size_t)__ldg(S.op_slot + o) * 32u + lane];
        st[(ps & 0xffff) * 32 + lane] -= lvv * st[(ps >> 16) * 32 + lane];
      }
      const T piv = st[ulen * 32 + lane];
      if (piv == (T)0) bad = true;
      T colmax = fabs(piv);
      for (int t = 0; t < llen; t++) colmax = fmax(colmax, fabs(st[(ulen + 1 + t) * 32 + lane]));
      if ((float)fabs(piv) < ptol * (float)colmax) tiny = true;
      const T inv = (T)1 / piv;
      T* dst = LU + luG + (size_t)base * 32u;
      if (st != dst) {
        for (int p = 0; p <= ulen; p++) dst[p * 32 + lane] = st[p * 32 + lane];
      }
      for (int t = 0; t < llen; t++) {
        const int p = ulen + 1 + t;
        dst[p * 32 + lane] = st[p * 32 + lane] * inv;
      }
    }
    __syncthreads();
  }
  __shared__ int flags[2][32];
  if (threadIdx.x < 64) (&flags[0][0])[threadIdx.x] = 0;
  __syncthreads();
  if (bad) atomicOr(&flags[0][lane], 1);
  if (tiny) atomicOr(&flags[1][lane], 1);
  __syncthreads();
  if (warp == 0) {
    if (flags[0][lane]) D.sing[s] = 1;
    if (flags[1][lane]) D.piv_flag[s] = 1;
  }
}

// ---------------------------------------------------------------------------
// K4: solve.  One CTA per group; phases = dependency levels of each BTF
// block's forward (L, with the off-diagonal terms of later blocks folded in)
// and backward (U) substitution, blocks in reverse order.
template <typename T>
__global__ void __launch_bounds__(256) k_solve(SchedDev S, BatchDev D) {
  const int g = blockIdx.x;
  if (!D.gact[g]) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int s = g * 32 + lane;
  const T* LU = (const T*)D.lu;
  const T* OFF = (const T*)D.off;
  const T* RHS = (const T*)D.rhs;
  T* X = (T*)D.sol;
  const size_t luG = (size_t)g * S.n_slots * 32u;
  const size_t xG = (size_t)g * S.n_u * 32u;
  bool bad = false;
  for (int ph = 0; ph < S.n_phases; ph++) {
    const int r0 = __ldg(S.ph_ptr + ph), r1 = __ldg(S.ph_ptr + ph + 1);
    const int kind = __ldg(S.ph_kind + ph);
    for (int q = r0 + warp; q < r1; q += nw) {
      const int k = __ldg(S.ph_rows + q);
      if (kind == 0) {
        T v = RHS[xG + (size_t)k * 32u + lane];
        const int tb = __ldg(S.fw_ptr + k), te = __ldg(S.fw_ptr + k + 1);
        for (int t = tb; t < te; t++) {
          const int sl = __ldg(S.fw_slot + t), j = __ldg(S.fw_col + t);
          const T c = (sl >= 0) ? LU[luG + (size_t)sl * 32u + lane]
                                : OFF[gidx(g, S.n_off, -sl - 1, lane)];
          v -= c * X[xG + (size_t)j * 32u + lane];
        }
        X[xG + (size_t)k * 32u + lane] = v;
      } else {
        T v = X[xG + (size_t)k * 32u + lane];
        const int tb = __ldg(S.bw_ptr + k), te = __ldg(S.bw_ptr + k + 1);
        for (int t = tb; t < te; t++) {
          const int sl = __ldg(S.bw_slot + t), j = __ldg(S.bw_col + t);
          v -= LU[luG + (size_t)sl * 32u + lane] * X[xG + (size_t)j * 32u + lane];
        }
        v = v / LU[luG + (size_t)__ldg(S.diag_slot + k) * 32u + lane];
        if (!isfinite((double)v)) bad = true;
        X[xG + (size_t)k * 32u + lane] = v;
      }
    }
    __syncthreads();
  }
  __shared__ int fl[32];
  if (threadIdx.x < 32) fl[threadIdx.x] = 0;
  __syncthreads();
  if (bad) atomicOr(&fl[lane], 1);
  __syncthreads();
  if (warp == 0 && fl[lane]) D.sing[s] = 1;
}

}  // namespace gox
