// CUDA kernels of the batched Newton-Raphson path (sm_103a).
//
// Lane l of a warp works on scenario 32*g + l of group g; all lanes run the
// same instruction stream on their own scenario's values, so every global
// access is one coalesced transaction (layout: gox_engine.hpp) and every
// schedule read is a warp-uniform broadcast.
//
//   k_update    K5 + K1a: apply the previous Newton step, V = |V| e^{j theta}
//   k_inject    K1b: S = V conj(Y V), mismatch F (FP64), per-scenario max|F|
//   k_decide    K1c: convergence / status / history per scenario
//   k_fill      K2: Jacobian values in the refactor's consumption order,
//               trig-free rectangular form (FP64 or FP32 out)
//   k_refactor  K3: level-synchronous left-looking refactorization with the
//               static pivot order (+ fused forward substitution)
//   k_solve     K4: row-oriented substitution phases
// The refactor and solve process one 32-scenario group per CTA and issue all
// independent loads of a column / row before any dependent arithmetic, so a
// dependency level costs one memory round trip.  No kernel waits on another
// CTA: only __syncthreads inside a CTA.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "gox_stream.hpp"

namespace gox {

enum : int { ST_RUNNING = -1, ST_CONVERGED = 0, ST_MAXITER = 1, ST_SINGULAR = 2, ST_UNUSED = 3 };

struct SchedDev {
  int n_bus, n_u, n_a, n_slots, n_off, n_levels, n_phases, nnz_y, fuse_fwd;
  int n_off_real;  // off-diagonal entries (n_off is at least 1 for allocation)
  const int32_t *yp, *yi;
  const double *yre, *yim;
  const int32_t *bus_rowP, *bus_rowQ, *bus_colA, *bus_colV;
  const int32_t *a_kind, *a_bi, *a_bk, *a_yslot, *a_dst;
  const int32_t *lev_ptr, *lev_cols, *c_base, *c_ulen, *c_llen, *c_abeg, *c_aend, *op_ptr, *op_slot;
  const uint32_t* op_pos;
  const int32_t* bt_ptr;
  const uint8_t* bt_cnt;
  const int32_t *pk_off, *pk;
  const int32_t *slot_a, *off_a;
  // fill tasks (one per Y entry with Jacobian entries): destinations of
  // H, N, M, L; {bus i, bus k, Y slot, diagonal}; Y's value (FP64, and
  // rounded to FP32 for the FP32 fill); then the zero fill-in slots
  int n_ftask, n_fzero;
  const int4 *ft_dst, *ft_bus;
  const double2* ft_y;
  const float2* ft_yf;
  const int32_t* fz_slot;
  const int32_t *ph_ptr, *ph_rows, *ph_kind, *fw_ptr, *fw_slot, *fw_col, *bw_ptr, *bw_slot,
      *bw_col, *diag_slot;
  // ZIP terms of the effective injection, or null: [4][n_bus] constant-
  // impedance re, im, constant-current re, im (per unit at |V| = 1)
  const double* zip;
};

// effective_injection (src/network.rs:600-611): s = p + jq, then + s_imp |V|
// |V| and + s_cur |V|, at the bus's present |V|
__device__ __forceinline__ double eff_inj(const double* zip, int nb, int i, int part, double s,
                                          double vm) {
  if (zip == nullptr) return s;
  s += zip[(size_t)part * nb + i] * vm * vm;
  s += zip[(size_t)(2 + part) * nb + i] * vm;
  return s;
}

struct BatchDev {
  int G;          // groups of 32 scenarios
  int max_iter;
  double tol;
  // FP64 state [G][n_bus][32]; cth, sth: cos / sin of va
  double *vm, *va, *e, *f, *psp, *qsp, *cth, *sth;
  // typed working arrays (T = float or double)
  void *eT, *fT, *ivT, *pT, *qT;  // [G][n_bus][32]
  void *jbuf;                      // [G][n_a][32]
  void *lu;                        // [G][n_slots][32]
  void *off;                       // [G][n_off][32]
  void *rhs, *sol;                 // [G][n_u][32]
  // per scenario [G*32]
  int32_t *status, *iters, *sing, *piv_flag;
  double *maxmis;
  unsigned long long* maxacc;      // max |F| of the running iteration (bits of a double >= 0)
  double *hist;                    // [G*32][max_iter] or null
  int32_t *gact;                   // [G] group has a running lane
  int32_t *nactive;                // [1] running groups after the last decision
  // optional per-scenario outage: 4 Y slots + deltas, and the branch buses
  const int32_t *o_slot, *o_bf, *o_bt;
  const double *o_dre, *o_dim;
  float piv_tol;                   // pivot-ratio threshold (mixed path)
  int32_t* err;                    // [0] set when a bounded device wait gave up
  int32_t* itp;                    // [1] iteration of the graph-captured loop (kernels given it < 0)
};

__device__ __forceinline__ size_t gidx(int g, int n, int e, int lane) {
  return ((size_t)g * (size_t)n + (size_t)e) * 32u + (size_t)lane;
}

// ---------------------------------------------------------------------------
// Conversions between FP64 and FP32 by integer operations.  This GPU runs
// a cvt between the two at the rate of an FP64 FMA, and the FP64 pipe is
// what bounds the mismatch kernels.
// f32_rn: round to nearest even (the value of (float)x) for results in the
// normal FP32 range; overflow gives infinity and NaN a quiet NaN, results
// below the smallest normal FP32 number (1.2e-38) become a zero of x's sign.
__device__ __forceinline__ float f32_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned ex = (hi >> 20) & 0x7ffu;
  const unsigned mant = ((hi & 0xfffffu) << 3) | (lo >> 29);  // top 23 fraction bits
  unsigned f = ((ex - 896u) << 23) + mant;
  const unsigned rem = lo & 0x1fffffffu;  // the 29 bits rounded off
  f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
  f = ex < 897u ? 0u : f;
  f = ex > 1150u ? 0x7f800000u : f;
  f = (ex == 2047u && ((hi & 0xfffffu) | lo) != 0u) ? 0x7fc00000u : f;
  return __uint_as_float(f | (hi & 0x80000000u));
}
// f64_of: the exact FP64 value of an FP32 number (FP32 subnormals, below
// 1.2e-38, become a zero of the same sign)
__device__ __forceinline__ double f64_of(float v) {
  const unsigned u = __float_as_uint(v);
  const unsigned ex = (u >> 23) & 0xffu;
  unsigned hi = ((ex + 896u) << 20) | ((u & 0x7fffffu) >> 3);
  hi = ex == 0u ? 0u : (ex == 255u ? (0x7ff00000u | ((u & 0x7fffffu) >> 3) | ((u & 0x7fffffu) ? 0x80000u : 0u)) : hi);
  const unsigned lo = ex == 0u ? 0u : (u << 29);
  return __longlong_as_double((long long)(((unsigned long long)(hi | (u & 0x80000000u)) << 32) | lo));
}
template <typename T>
__device__ __forceinline__ T to_T(double x) {
  if constexpr (sizeof(T) == 4) return f32_rn(x);
  else return x;
}
template <typename T>
__device__ __forceinline__ double from_T(T v) {
  if constexpr (sizeof(T) == 4) return f64_of(v);
  else return v;
}

// ---------------------------------------------------------------------------
// K5 + K1a.  grid (ceil(N/8), G), 8 warps: warp -> bus, lane -> scenario.
// mode 0: iteration `it`; mode 1: the update after the last iteration.
template <typename T>
__device__ __forceinline__ void update_body(const SchedDev& S, const BatchDev& D, int it, int mode,
                                            int BX, int BY) {
  if (it < 0) it = *D.itp;
  const int g = BY;
  const int lane = threadIdx.x & 31;
  const int i = BX * 8 + (threadIdx.x >> 5);
  const int N = S.n_bus;
  // a block is 8 warps (a wider CTA's other warps take no part)
  if (i >= N || (threadIdx.x >> 5) >= 8) return;
  const int s = g * 32 + lane;
  const bool upd = D.status[s] == ST_RUNNING && (it > 0 || mode == 1) && D.sing[s] == 0;
  const size_t x = gidx(g, N, i, lane);
  double vm = D.vm[x], va = D.va[x];
  double dth = 0.0;
  float step = 0.0f;  // the angle step as solved (FP32 path): picks the formula below
  if (upd) {
    const T* sol = (const T*)D.sol;
    const int ca = __ldg(S.bus_colA + i), cv = __ldg(S.bus_colV + i);
    if (ca >= 0) {
      const T sa = sol[gidx(g, S.n_u, ca, lane)];
      if constexpr (sizeof(T) == 4) step = sa;
      const double va1 = va + from_T<T>(sa);
      dth = va1 - va;
      va = va1;
    }
    if (cv >= 0) vm += from_T<T>(sol[gidx(g, S.n_u, cv, lane)]);
    D.vm[x] = vm;
    D.va[x] = va;
  }
  if (mode != 0) return;
  // cos / sin of the angle: at the first iteration and after a large step
  // from sincos; after a small step (|d| < 1/32) by rotating the previous
  // pair by d, with cos d and sin d from their Taylor series (the first
  // omitted terms are below 1e-19 there; the rotation adds about one
  // rounding per iteration).  After a step below 2^-10 (the later
  // iterations) two terms of each series suffice (the first omitted ones are
  // below 2e-21).  The choice is each lane's own, so a scenario's rounding
  // does not depend on the other scenarios of its group (re-packing moves
  // scenarios between groups).
  // (the FP32 path compares the step as solved: an FP32 compare)
  double sn, cs;
  const float ad = sizeof(T) == 4 ? fabsf(step) : 0.0f;
  const bool small = it > 0 && (sizeof(T) == 4 ? ad < 0.03125f : fabs(dth) < 0.03125);
  const bool tiny = it > 0 && (sizeof(T) == 4 ? ad < 0.0009765625f : fabs(dth) < 0.0009765625);
  if (tiny) {
    const double d2 = dth * dth;
    const double cd = 1.0 + d2 * (-1.0 / 2 + d2 * (1.0 / 24));
    const double sd = dth * (1.0 + d2 * (-1.0 / 6 + d2 * (1.0 / 120)));
    const double c0 = D.cth[x], s0 = D.sth[x];
    cs = c0 * cd - s0 * sd;
    sn = s0 * cd + c0 * sd;
  } else if (small) {
    const double d2 = dth * dth;
    const double cd = 1.0 + d2 * (-1.0 / 2 + d2 * (1.0 / 24 + d2 * (-1.0 / 720 + d2 * (1.0 / 40320))));
    const double sd = dth * (1.0 + d2 * (-1.0 / 6 + d2 * (1.0 / 120 + d2 * (-1.0 / 5040))));
    const double c0 = D.cth[x], s0 = D.sth[x];
    cs = c0 * cd - s0 * sd;
    sn = s0 * cd + c0 * sd;
  } else {
    sincos(va, &sn, &cs);
  }
  D.cth[x] = cs;
  D.sth[x] = sn;
  const double e = vm * cs, f = vm * sn;
  D.e[x] = e;
  D.f[x] = f;
  ((T*)D.eT)[x] = to_T<T>(e);
  ((T*)D.fT)[x] = to_T<T>(f);
  // 1/|V| for the Jacobian fill, in the fill's precision (an FP64 division
  // costs far more than an FP32 one on this GPU)
  ((T*)D.ivT)[x] = (T)1 / to_T<T>(vm);
}
template <typename T>
__global__ void __launch_bounds__(256) k_update(SchedDev S, BatchDev D, int it, int mode) {
  update_body<T>(S, D, it, mode, blockIdx.x, blockIdx.y);
}

// ---------------------------------------------------------------------------
// K1b: S = V conj(Y V), F, max|F|.  grid (ceil(N / (8*BPW)), G), 8 warps,
// each warp BPW consecutive buses.  FP64 instructions are the cost of this
// kernel (the GPU runs them at 1/64 of the FP32 rate, and an instruction
// whose predicate is false for every lane still takes its issue slot), so a
// row of Y runs exactly its entries: a warp-uniform switch on the row's
// length into a fully unrolled body that issues its L neighbour loads
// before its 4 L FMAs.  max|F| is kept as the bit pattern of |F| (ordered
// like the value for non-negative doubles) by integer max, NaN skipped as
// fmax does.
template <int L>
__device__ __forceinline__ void y_row(const SchedDev& S, const double* __restrict__ e,
                                      const double* __restrict__ f, int g, int N, int lane,
                                      int p, double& ir, double& ii) {
  double ek[L], fk[L], gr[L], gi[L];
#pragma unroll
  for (int t = 0; t < L; t++) {
    const int k = __ldg(S.yi + p + t);
    gr[t] = __ldg(S.yre + p + t);
    gi[t] = __ldg(S.yim + p + t);
    const size_t xk = gidx(g, N, k, lane);
    ek[t] = e[xk];
    fk[t] = f[xk];
  }
#pragma unroll
  for (int t = 0; t < L; t++) {
    ir = fma(gr[t], ek[t], ir);
    ir = fma(-gi[t], fk[t], ir);
    ii = fma(gr[t], fk[t], ii);
    ii = fma(gi[t], ek[t], ii);
  }
}

__device__ __forceinline__ unsigned long long abs_bits(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
  return b > 0x7ff0000000000000ull ? 0ull : b;  // NaN: skipped
}

template <typename T, bool OUTAGE, int BPW, bool ZIP>
__device__ __forceinline__ void inject_body(const SchedDev& S, const BatchDev& D, int it, int BX,
                                            int BY) {
  if (it < 0) it = *D.itp;
  const int g = BY;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int s = g * 32 + lane;
  const int N = S.n_bus;
  __shared__ unsigned long long red[8][32];
  const bool active = D.status[s] == ST_RUNNING && !(it > 0 && D.sing[s] != 0);
  T* rhs = (T*)D.rhs;
  const double* __restrict__ e = D.e;
  const double* __restrict__ f = D.f;
  int obf = -1, obt = -1;
  if (OUTAGE) { obf = D.o_bf[s]; obt = D.o_bt[s]; }
  unsigned long long mx = 0ull;
  // a block is 8 warps; a wider CTA's other warps only take its barrier
  const bool in_block = warp < 8;
  const int i0 = in_block ? (BX * 8 + warp) * BPW : N;
  for (int i = i0; i < min(N, i0 + BPW); i++) {
    double ir = 0.0, ii = 0.0;
    int p = __ldg(S.yp + i);
    const int pe = __ldg(S.yp + i + 1);
    while (pe - p > 8) {
      y_row<8>(S, e, f, g, N, lane, p, ir, ii);
      p += 8;
    }
    switch (pe - p) {
      case 1: y_row<1>(S, e, f, g, N, lane, p, ir, ii); break;
      case 2: y_row<2>(S, e, f, g, N, lane, p, ir, ii); break;
      case 3: y_row<3>(S, e, f, g, N, lane, p, ir, ii); break;
      case 4: y_row<4>(S, e, f, g, N, lane, p, ir, ii); break;
      case 5: y_row<5>(S, e, f, g, N, lane, p, ir, ii); break;
      case 6: y_row<6>(S, e, f, g, N, lane, p, ir, ii); break;
      case 7: y_row<7>(S, e, f, g, N, lane, p, ir, ii); break;
      case 8: y_row<8>(S, e, f, g, N, lane, p, ir, ii); break;
      default: break;
    }
    const size_t x = gidx(g, N, i, lane);
    const double ei = e[x], fi = f[x];
    if (OUTAGE && (i == obf || i == obt)) {
      const size_t xf = gidx(g, N, obf, lane), xt = gidx(g, N, obt, lane);
      const double ef = e[xf], ff = f[xf], et = e[xt], ft = f[xt];
      const int c0 = (i == obf) ? 0 : 2;
      const double ar = D.o_dre[4 * s + c0], ai = D.o_dim[4 * s + c0];
      const double br = D.o_dre[4 * s + c0 + 1], bi = D.o_dim[4 * s + c0 + 1];
      ir += ar * ef - ai * ff + br * et - bi * ft;
      ii += ar * ff + ai * ef + br * ft + bi * et;
    }
    const int rp = __ldg(S.bus_rowP + i), rq = __ldg(S.bus_rowQ + i);
    if constexpr (sizeof(T) == 4) {
      // F = S_spec - V conj(I) in FP64 as two FMAs per component; the FP32
      // Jacobian's P and Q are S_spec - F in FP32 (only the buses with a P
      // row have Jacobian entries that use them; a PV bus's Q comes from
      // the products, it has no Q row)
      if (rp >= 0) {
        const double psp = ZIP ? eff_inj(S.zip, N, i, 0, D.psp[x], D.vm[x]) : D.psp[x];
        const double FP = fma(-fi, ii, fma(-ei, ir, psp));
        const float fp = f32_rn(FP);
        if (active) {
          mx = max(mx, abs_bits(FP));
          rhs[gidx(g, S.n_u, rp, lane)] = fp;
        }
        ((float*)D.pT)[x] = f32_rn(psp) - fp;
        if (rq >= 0) {
          const double qsp = ZIP ? eff_inj(S.zip, N, i, 1, D.qsp[x], D.vm[x]) : D.qsp[x];
          const double FQ = fma(ei, ii, fma(-fi, ir, qsp));
          const float fq = f32_rn(FQ);
          if (active) {
            mx = max(mx, abs_bits(FQ));
            rhs[gidx(g, S.n_u, rq, lane)] = fq;
          }
          ((float*)D.qT)[x] = f32_rn(qsp) - fq;
        } else {
          ((float*)D.qT)[x] = f32_rn(fi * ir - ei * ii);
        }
      }
    } else {
      const double pc = ei * ir + fi * ii;
      const double qc = fi * ir - ei * ii;
      if (active) {
        if (rp >= 0) {
          const double F = (ZIP ? eff_inj(S.zip, N, i, 0, D.psp[x], D.vm[x]) : D.psp[x]) - pc;
          mx = max(mx, abs_bits(F));
          rhs[gidx(g, S.n_u, rp, lane)] = (T)F;
        }
        if (rq >= 0) {
          const double F = (ZIP ? eff_inj(S.zip, N, i, 1, D.qsp[x], D.vm[x]) : D.qsp[x]) - qc;
          mx = max(mx, abs_bits(F));
          rhs[gidx(g, S.n_u, rq, lane)] = (T)F;
        }
      }
      ((T*)D.pT)[x] = (T)pc;
      ((T*)D.qT)[x] = (T)qc;
    }
  }
  if (in_block) red[warp][lane] = mx;
  __syncthreads();
  if (warp == 0) {
    unsigned long long m = 0ull;
#pragma unroll
    for (int w = 0; w < 8; w++) m = max(m, red[w][lane]);
    if (active && m > 0ull) atomicMax(D.maxacc + s, m);
  }
}
template <typename T, bool OUTAGE, int BPW, bool ZIP>
__global__ void __launch_bounds__(256) k_inject(SchedDev S, BatchDev D, int it) {
  inject_body<T, OUTAGE, BPW, ZIP>(S, D, it, blockIdx.x, blockIdx.y);
}

__device__ __forceinline__ void decide_body(const BatchDev& D, int it, int mode, int BX) {
  if (it < 0) it = *D.itp;
  const int g = BX, lane = threadIdx.x;
  const int s = g * 32 + lane;
  bool running = D.status[s] == ST_RUNNING;
  if (running) {
    const int sg = D.sing[s];
    if ((it > 0 || mode == 1) && sg != 0) {
      D.status[s] = ST_SINGULAR;  // Singular: the previous solve failed, V untouched
      running = false;
    } else if (mode == 1) {
      D.status[s] = ST_MAXITER;
      running = false;
    } else {
      const double m = __longlong_as_double((long long)D.maxacc[s]);
      D.maxmis[s] = m;
      if (D.hist) D.hist[(size_t)s * D.max_iter + it] = m;
      D.iters[s] = it + 1;
      D.sing[s] = (sg == 2) ? 2 : 0;  // 2: the scenario's own first factorization failed
      if (m < D.tol) {
        D.status[s] = ST_CONVERGED;
        running = false;
      }
    }
  }
  D.maxacc[s] = 0ull;
  const unsigned any = __ballot_sync(0xffffffffu, running);
  if (lane == 0) {
    D.gact[g] = any ? 1 : 0;
    if (any) atomicAdd(D.nactive, 1);
  }
}
__global__ void k_decide(BatchDev D, int it, int mode) { decide_body(D, it, mode, blockIdx.x); }

// The graph-captured Newton loop's decision, one thread after k_decide: run
// this iteration's Jacobian, refactor and solves while a scenario is running
// (hif), iterate again while one is and the budget allows (hw), or evaluate
// the final MaxIterations mismatch when the budget is spent (hmax).
__global__ void k_cond(const int32_t* __restrict__ nactive, int32_t* itp, int max_iter,
                       cudaGraphConditionalHandle hw, cudaGraphConditionalHandle hif,
                       cudaGraphConditionalHandle hmax) {
  const unsigned any = *nactive > 0 ? 1u : 0u;
  const int next = *itp + 1;
  cudaGraphSetConditional(hif, any);
  cudaGraphSetConditional(hw, any && next < max_iter ? 1u : 0u);
  cudaGraphSetConditional(hmax, any && next >= max_iter ? 1u : 0u);
  *itp = next;
}

// ---------------------------------------------------------------------------
// K2: Jacobian fill (src/jacobian.rs:202-250 formulas in rectangular form:
// V_i V_k cos(th_i - th_k) = e_i e_k + f_i f_k, V_i V_k sin(..) = f_i e_k - e_i f_k),
// written straight into the factor's layout, so the refactor starts a
// column with one copy of its rows.  One task per Y entry (i, k) that has
// Jacobian entries: its four entries H, N, M, L share the bus values and
// the products, so a task loads five rows and stores up to four (entries
// absent from the Jacobian have destination -1).  A destination below
// n_slots is an LU slot, else an off-diagonal (BTF) entry.  The fill-in
// slots of the factor are zeroed by the last warps, four rows (FP32) per
// 16-byte store.  grid (chunks, G): warps [0, tw) run `per_warp` tasks
// each, the others zero 32 slots each.
template <typename T>
__device__ __forceinline__ void fill_store(T* LU, T* OFF, int n_slots, int x, int lane, T v) {
  if (x < 0) return;
  if (x < n_slots) LU[(size_t)x * 32u + lane] = v;
  else OFF[(size_t)(x - n_slots) * 32u + lane] = v;
}

template <typename T, bool OUTAGE>
__device__ __forceinline__ void fill_body(const SchedDev& S, const BatchDev& D, int tw, int per_warp,
                                          int BX, int BY) {
  const int g = BY;
  if (!D.gact[g] || (threadIdx.x >> 5) >= 8) return;  // a block is 8 warps
  const int lane = threadIdx.x & 31;
  const int wglob = BX * 8 + (threadIdx.x >> 5);
  const int N = S.n_bus;
  T* LU = (T*)D.lu + (size_t)g * S.n_slots * 32u;
  T* OFF = (T*)D.off + (size_t)g * S.n_off * 32u;
  if (wglob >= tw) {
    // zero fill-in slots: lanes of a 16-byte store cover one row
    constexpr int LPR = 32 * (int)sizeof(T) / 16;  // lanes per row
    constexpr int RPI = 32 / LPR;                  // rows per store
    const int z0 = (wglob - tw) * 32;
    const int sub = lane % LPR;
#pragma unroll
    for (int q = 0; q < 32; q += RPI) {
      const int z = z0 + q + lane / LPR;
      if (z < S.n_fzero) {
        const int x = __ldg(S.fz_slot + z);
        *reinterpret_cast<float4*>(reinterpret_cast<char*>(LU + (size_t)x * 32u) + sub * 16) =
            make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    return;
  }
  const int t0 = wglob * per_warp;
  if (t0 >= S.n_ftask) return;
  const int t1 = min(S.n_ftask, t0 + per_warp);
  const int s = g * 32 + lane;
  const size_t gb = (size_t)g * N * 32u + lane;
  const T* eT = (const T*)D.eT + gb;
  const T* fT = (const T*)D.fT + gb;
  const T* ivT = (const T*)D.ivT + gb;
  const T* pT = (const T*)D.pT + gb;
  const T* qT = (const T*)D.qT + gb;
  int os0 = -1, os1 = -1, os2 = -1, os3 = -1;
  if (OUTAGE && D.o_bf[s] >= 0) {
    os0 = D.o_slot[4 * s]; os1 = D.o_slot[4 * s + 1]; os2 = D.o_slot[4 * s + 2]; os3 = D.o_slot[4 * s + 3];
  }
  constexpr int U = 2;  // tasks in flight per warp (2: 48 registers, more warps per SM than 4 in flight)
  for (int ta = t0; ta < t1; ta += U) {
    int4 dst[U], bus[U];
    T G[U], B[U], v[U][5];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int t = min(ta + u, t1 - 1);
      dst[u] = __ldg(S.ft_dst + t);
      bus[u] = __ldg(S.ft_bus + t);
      if constexpr (sizeof(T) == 4) {
        // FP32 fill: Y rounded once on the host (a conversion per value here
        // would run on the FP64 pipe)
        const float2 y = __ldg(S.ft_yf + t);
        G[u] = y.x;
        B[u] = y.y;
      } else {
        const double2 y = __ldg(S.ft_y + t);
        G[u] = y.x;
        B[u] = y.y;
      }
      // five rows: e_i, f_i and (diagonal) 1/|V_i|, P_i, Q_i or
      // (off-diagonal) e_k, f_k, 1/|V_k|
      const size_t xi = (size_t)bus[u].x * 32u, xk = (size_t)bus[u].y * 32u;
      const bool dg = bus[u].w != 0;
      v[u][0] = eT[xi];
      v[u][1] = fT[xi];
      v[u][2] = dg ? ivT[xi] : eT[xk];
      v[u][3] = dg ? pT[xi] : fT[xk];
      v[u][4] = dg ? qT[xi] : ivT[xk];
    }
    if (OUTAGE) {
      // the outaged branch's Y entries: Y + delta in FP64, then rounded
      // (the warp takes this branch only when one of its lanes needs it)
#pragma unroll
      for (int u = 0; u < U; u++) {
        const int ys = bus[u].z;
        const int c = (ys == os0) ? 0 : (ys == os1) ? 1 : (ys == os2) ? 2 : (ys == os3) ? 3 : -1;
        if (__any_sync(0xffffffffu, c >= 0)) {
          if (c >= 0) {
            const double2 y = __ldg(S.ft_y + min(ta + u, t1 - 1));
            G[u] = (T)(y.x + D.o_dre[4 * s + c]);
            B[u] = (T)(y.y + D.o_dim[4 * s + c]);
          }
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (ta + u >= t1) break;
      T h, nn, m, l;
      if (bus[u].w != 0) {
        const T ei = v[u][0], fi = v[u][1], iv = v[u][2], P = v[u][3], Q = v[u][4];
        const T vi2 = ei * ei + fi * fi;
        const T vi = vi2 * iv;  // |V_i|^2 / |V_i|
        h = -Q - vi2 * B[u];       // H_ii
        nn = P * iv + vi * G[u];   // N_ii
        m = P - vi2 * G[u];        // M_ii
        l = Q * iv - vi * B[u];    // L_ii
      } else {
        const T ei = v[u][0], fi = v[u][1], ek = v[u][2], fk = v[u][3], ivk = v[u][4];
        const T c = ei * ek + fi * fk;   // V_i V_k cos
        const T sn = fi * ek - ei * fk;  // V_i V_k sin
        const T a = G[u] * sn - B[u] * c;
        const T b = G[u] * c + B[u] * sn;
        h = a;          // H_ik
        nn = b * ivk;   // N_ik
        m = -b;         // M_ik
        l = a * ivk;    // L_ik
      }
      fill_store(LU, OFF, S.n_slots, dst[u].x, lane, h);
      fill_store(LU, OFF, S.n_slots, dst[u].y, lane, nn);
      fill_store(LU, OFF, S.n_slots, dst[u].z, lane, m);
      fill_store(LU, OFF, S.n_slots, dst[u].w, lane, l);
    }
  }
}
template <typename T, bool OUTAGE>
__global__ void __launch_bounds__(256) k_fill(SchedDev S, BatchDev D, int tw, int per_warp) {
  fill_body<T, OUTAGE>(S, D, tw, per_warp, blockIdx.x, blockIdx.y);
}

// Bulk (TMA) copy global -> shared with mbarrier completion, and a bounded
// wait on it: after kSpinLimit polls the wait gives up and reports false.
constexpr int kSpinLimit = 1 << 22;
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "fence.proxy.async.shared::cta;\n"
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%2], %3;\n"
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %3, [%2];\n"
      ::"r"(smem_u32(dst)), "l"(src), "r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  const unsigned a = smem_u32(bar);
  for (int it = 0; it < kSpinLimit; it++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done) : "r"(a), "r"(parity) : "memory");
    if (done) return true;
  }
  return false;
}

// Shared-memory accesses by 32-bit shared address (the ring and the stage
// are addressed by row numbers computed at run time).
template <typename T>
__device__ __forceinline__ T lds(uint32_t a);
template <>
__device__ __forceinline__ float lds<float>(uint32_t a) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1];\n" : "=f"(v) : "r"(a));
  return v;
}
template <>
__device__ __forceinline__ double lds<double>(uint32_t a) {
  double v;
  asm volatile("ld.shared.f64 %0, [%1];\n" : "=d"(v) : "r"(a));
  return v;
}
// ... with a compile-time byte offset folded into the instruction
template <typename T, int OFF>
__device__ __forceinline__ T lds_off(uint32_t a);
template <>
__device__ __forceinline__ float lds_off<float, 0>(uint32_t a) { return lds<float>(a); }
#define GOX_LDS_OFF(TY, PT, CT, OFFV)                                                  \
  template <>                                                                     \
  __device__ __forceinline__ TY lds_off<TY, OFFV>(uint32_t a) {                    \
    TY v;                                                                         \
    asm volatile("ld.shared." PT " %0, [%1+" #OFFV "];\n" : "=" CT(v) : "r"(a));     \
    return v;                                                                     \
  }
GOX_LDS_OFF(float, "f32", "f", 128)
GOX_LDS_OFF(float, "f32", "f", 256)
GOX_LDS_OFF(float, "f32", "f", 384)
GOX_LDS_OFF(float, "f32", "f", 512)
GOX_LDS_OFF(float, "f32", "f", 640)
GOX_LDS_OFF(float, "f32", "f", 768)
GOX_LDS_OFF(float, "f32", "f", 896)
GOX_LDS_OFF(float, "f32", "f", 1024)
#undef GOX_LDS_OFF
__device__ __forceinline__ void sts(uint32_t a, float v) {
  asm volatile("st.shared.f32 [%0], %1;\n" ::"r"(a), "f"(v) : "memory");
}
__device__ __forceinline__ void sts(uint32_t a, double v) {
  asm volatile("st.shared.f64 [%0], %1;\n" ::"r"(a), "d"(v) : "memory");
}
__device__ __forceinline__ uint4 lds128(uint32_t a) {
  uint4 v;
  asm volatile("ld.shared.v4.b32 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "r"(a)
               : "memory");
  return v;
}
__device__ __forceinline__ void cp_async16(uint32_t smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(smem), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_n(int n) {
  switch (n) {
    case 0: asm volatile("cp.async.wait_group 0;\n" ::: "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;\n" ::: "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;\n" ::: "memory"); break;
    case 3: asm volatile("cp.async.wait_group 3;\n" ::: "memory"); break;
    case 4: asm volatile("cp.async.wait_group 4;\n" ::: "memory"); break;
    case 5: asm volatile("cp.async.wait_group 5;\n" ::: "memory"); break;
    case 6: asm volatile("cp.async.wait_group 6;\n" ::: "memory"); break;
    default: asm volatile("cp.async.wait_group 7;\n" ::: "memory"); break;
  }
}

// Correctly rounded reciprocal (the same value as 1 / x).
__device__ __forceinline__ float rcp_rn(float x) { return __frcp_rn(x); }
__device__ __forceinline__ double rcp_rn(double x) { return __drcp_rn(x); }

// The refactor's command streams on the device (built on the host: one
// stream per warp, in chunks of chunk_words words).
struct StreamDev {
  const int32_t* words;
  const int32_t* chunk0;
  const int32_t* nchunks;
  int ring_rows, chunk_words, n_bars;
  int rows_total;  // rows of all rings (the zero row follows them)
  int sync;        // levels end in: 0 CTA barriers, 1 per-warp progress flags
};

// Progress flags (plans with sync = 1).  A warp that has done its work of
// the first n levels publishes n: every lane fences its shared and global
// writes (and the copies it waited for) at CTA scope, the warp meets, and
// lane 0 stores n with release semantics.  A warp waits for another's count
// with acquire loads by all lanes, a bounded number of polls, and gives up
// early once any warp of the CTA has failed.
__device__ __forceinline__ void publish_level(int* prog, int warp, int lane, int n) {
  __threadfence_block();
  __syncwarp();
  if (lane == 0)
    asm volatile("st.release.cta.shared.b32 [%0], %1;\n" ::"r"(smem_u32(prog + warp)), "r"(n)
                 : "memory");
}
__device__ __forceinline__ int ld_acquire_s32(const int* p) {
  int v;
  asm volatile("ld.acquire.cta.shared.b32 %0, [%1];\n" : "=r"(v) : "r"(smem_u32(p)) : "memory");
  return v;
}
// m words v | n << 8 (warp v has published n levels); false when a wait gave up
__device__ __forceinline__ bool wait_levels(const int32_t* w, int m, const int* prog,
                                            const volatile int* failed) {
  for (int q = 0; q < m; q++) {
    const int v = w[q] & 0xff, need = (int)(((uint32_t)w[q]) >> 8);
    for (int it = 0; !__all_sync(0xffffffffu, ld_acquire_s32(prog + v) >= need); it++)
      if (__any_sync(0xffffffffu, it >= kSpinLimit || *failed != 0)) return false;
  }
  return true;
}

// Pieces of the refactor interpreter.  Every loop below runs over counts the
// stream compiler padded (gather rows to 2 copies, steps to pairs, forward
// terms to 8), so no branch depends on a value inside an iteration.
template <typename T>
struct Rf {
  static constexpr uint32_t RB = 32u * sizeof(T);  // bytes per row
  static constexpr int RPI = 512 / (int)RB;        // rows per 16-byte-per-lane copy
  static constexpr int LPR = 32 / RPI;             // lanes per row in a copy

  // m rows (multiple of 2 * RPI): words src_row | dst_row << 21 over the row
  // space [factor image | X | right-hand side]
  static __device__ __forceinline__ void gather(const int32_t* w, int m, uint32_t ring_s, int lane,
                                                const T* LUg, const T* Xg, const T* RHSg,
                                                int n_slots, int n_u) {
    const int sub = lane % LPR, rsel = lane / LPR;
    for (int q0 = 0; q0 < m; q0 += 2 * RPI) {
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const uint32_t rw = (uint32_t)w[q0 + h * RPI + rsel];
        const uint32_t v = rw & 0x1fffffu;
        const char* src = v < (uint32_t)n_slots ? (const char*)LUg + (size_t)v * RB
                          : v < (uint32_t)(n_slots + n_u)
                              ? (const char*)Xg + (size_t)(v - n_slots) * RB
                              : (const char*)RHSg + (size_t)(v - n_slots - n_u) * RB;
        cp_async16(ring_s + (rw >> 21) * RB + (uint32_t)sub * 16u, src + (size_t)sub * 16u);
      }
    }
  }

  // One step: 9 updates stage[d] -= L(d, j) * stage[j].  FP32 runs all 9
  // (unused ones on the dummy row: no branch); FP64 skips the unused ones,
  // since an FP64 FMA costs far more than a uniform branch on this GPU.
  static __device__ __forceinline__ void step(uint4 d, uint32_t st_lane, uint32_t ring_lane) {
    const uint32_t la = ring_lane + (d.x & 0xffffu) * RB;
    const T xj = lds<T>(st_lane + ((d.x >> 16) & 0x3ffu) * RB);
    uint32_t da[kStepOps];
    T xi[kStepOps], lv[kStepOps];
#pragma unroll
    for (int t = 0; t < kStepOps; t++) {
      const uint32_t wd = t < 3 ? d.y : (t < 6 ? d.z : d.w);
      da[t] = st_lane + ((wd >> (10 * (t % 3))) & 0x3ffu) * RB;
    }
    if (sizeof(T) == 4) {
      load_l<0>(la, lv);
#pragma unroll
      for (int t = 0; t < kStepOps; t++) xi[t] = lds<T>(da[t]);
#pragma unroll
      for (int t = 0; t < kStepOps; t++) sts(da[t], xi[t] - lv[t] * xj);
    } else {
      const int cnt = (int)(d.x >> 26);
#pragma unroll
      for (int t = 0; t < kStepOps; t++)
        if (t < cnt) {
          xi[t] = lds<T>(da[t]);
          lv[t] = lds<T>(la + (uint32_t)t * RB);
        }
#pragma unroll
      for (int t = 0; t < kStepOps; t++)
        if (t < cnt) sts(da[t], xi[t] - lv[t] * xj);
    }
  }
  // the 9 L values of a step (FP32: offsets folded into the loads)
  template <int Z>
  static __device__ __forceinline__ void load_l(uint32_t la, T* lv) {
    if constexpr (sizeof(T) == 4) {
      lv[0] = lds_off<float, 0>(la);
      lv[1] = lds_off<float, 128>(la);
      lv[2] = lds_off<float, 256>(la);
      lv[3] = lds_off<float, 384>(la);
      lv[4] = lds_off<float, 512>(la);
      lv[5] = lds_off<float, 640>(la);
      lv[6] = lds_off<float, 768>(la);
      lv[7] = lds_off<float, 896>(la);
      lv[8] = lds_off<float, 1024>(la);
    }
  }

  // m steps (even), uint4 each; the word after the last pair is readable
  static __device__ __forceinline__ void steps(const uint4* sd, int m, uint32_t st_lane,
                                               uint32_t ring_lane) {
    uint4 d0 = sd[0], d1 = sd[1];
    for (int q = 0; q < m; q += 2) {
      const uint4 n0 = sd[q + 2], n1 = sd[q + 3];
      step(d0, st_lane, ring_lane);
      step(d1, st_lane, ring_lane);
      d0 = n0;
      d1 = n1;
    }
  }

  // y = (first ? b : y) - sum L(k, j) y_j over m terms (multiple of 8; mr
  // of them real, the rest read the zero row; FP64 skips those)
  static __device__ __forceinline__ void fwd(const int32_t* w, int m, int mr, bool first,
                                             uint32_t yrow, uint32_t ring_lane) {
    T y = lds<T>(first ? yrow + RB : yrow);
    for (int f0 = 0; f0 < m; f0 += 8) {
      T a[8], b[8];
#pragma unroll
      for (int t = 0; t < 8; t++) {
        const uint32_t fw = (uint32_t)w[f0 + t];
        a[t] = lds<T>(ring_lane + (fw & 0xffffu) * RB);
        b[t] = lds<T>(ring_lane + (fw >> 16) * RB);
      }
      if (sizeof(T) == 4) {
#pragma unroll
        for (int t = 0; t < 8; t++) y -= a[t] * b[t];
      } else {
#pragma unroll
        for (int t = 0; t < 8; t++)
          if (f0 + t < mr) y -= a[t] * b[t];
      }
    }
    sts(yrow, y);
  }

  // x_k = (y_k - sum U(k, j) x_j) / U(k, k) over m terms (multiple of 8,
  // mr real; FP64 skips the padding); x_k to its row and to X
  static __device__ __forceinline__ void bwd(const int32_t* w, int m, int mr, uint32_t xrow,
                                             uint32_t yrow, uint32_t drow, uint32_t ring_lane,
                                             T* xg, bool& bad) {
    T v = lds<T>(yrow);
    for (int f0 = 0; f0 < m; f0 += 8) {
      T a[8], b[8];
#pragma unroll
      for (int t = 0; t < 8; t++) {
        const uint32_t fw = (uint32_t)w[f0 + t];
        a[t] = lds<T>(ring_lane + (fw & 0xffffu) * RB);
        b[t] = lds<T>(ring_lane + (fw >> 16) * RB);
      }
      if (sizeof(T) == 4) {
#pragma unroll
        for (int t = 0; t < 8; t++) v -= a[t] * b[t];
      } else {
#pragma unroll
        for (int t = 0; t < 8; t++)
          if (f0 + t < mr) v -= a[t] * b[t];
      }
    }
    const T x = v / lds<T>(drow);
    bad |= !isfinite(x);
    sts(xrow, x);
    *xg = x;
  }

  // pivot, scale L in place (each lane its scenario's rows, in blocks of 8,
  // the last block clamped to the column's end), then the column's rows to
  // its slots: a row of 32 values is contiguous both in the stage and in the
  // factor image, so each lane moves 16 bytes of one row per instruction
  static __device__ __forceinline__ void finish(int k, int base, int ulen, int llen, uint32_t st_lane,
                                                T* LUg, T* Xg, int lane, bool fuse, float ptol,
                                                bool& bad, bool& tiny) {
    const int len = ulen + 1 + llen;
    const T piv = lds<T>(st_lane + (uint32_t)ulen * RB);
    bad |= (piv == (T)0);
    const T inv = rcp_rn(piv);
    T colmax = fabs(piv);
    for (int p0 = ulen + 1; p0 < len; p0 += 8) {
      T v[8];
#pragma unroll
      for (int t = 0; t < 8; t++) v[t] = lds<T>(st_lane + (uint32_t)min(p0 + t, len - 1) * RB);
#pragma unroll
      for (int t = 0; t < 8; t++) colmax = fmax(colmax, fabs(v[t]));
#pragma unroll
      for (int t = 0; t < 8; t++) {
        if (sizeof(T) == 8 && p0 + t >= len) break;  // FP64: no duplicate multiplies
        v[t] *= inv;
        sts(st_lane + (uint32_t)min(p0 + t, len - 1) * RB, v[t]);
      }
    }
    tiny |= (ptol > 0.0f) && ((float)fabs(piv) < ptol * (float)colmax);
    if (fuse) Xg[(size_t)k * 32u + lane] = lds<T>(st_lane + (uint32_t)len * RB);
    __syncwarp();
    const int sub = lane % LPR, rsel = lane / LPR;
    const uint32_t blk = st_lane - (uint32_t)lane * (uint32_t)sizeof(T) + (uint32_t)sub * 16u;
    char* dst = reinterpret_cast<char*>(LUg + (size_t)base * 32u) + sub * 16;
    for (int r0 = rsel; r0 < len + rsel; r0 += 4 * RPI) {
      uint4 v[4];
#pragma unroll
      for (int u = 0; u < 4; u++) v[u] = lds128(blk + (uint32_t)min(r0 + u * RPI, len - 1) * RB);
#pragma unroll
      for (int u = 0; u < 4; u++)
        *reinterpret_cast<uint4*>(dst + (size_t)min(r0 + u * RPI, len - 1) * RB) = v[u];
    }
    __syncwarp();
  }
};

// K3: refactor, the interpreter of the per-warp command streams.  One CTA
// per group of 32 scenarios (lane = scenario).  Shared memory: per warp two
// stream chunks (TMA bulk copies, mbarrier completion, bounded waits), then
// the rings of all warps as one space of rows of 32 values, then the zero
// row, the trash row and spare rows.  The host has placed every value: a
// column's stage block holds [column rows | y | b | dummy]; update runs
// L(:, j) are read either from a copy in the warp's ring or straight from
// the producing column's block.  The common case of a column is one COLUMN
// command (copies for this column, copies issued ahead for the warp's next
// column, wait, update steps, forward-substitution terms, finish, optional
// level barrier); the single commands GATHER, WAIT, STEPS, FWD, FINISH,
// BAR cover columns whose values are fetched in pieces.  Every branch is
// per command or per loop trip; a step always performs 9 updates (unused
// ones on the block's dummy row).  A bounded wait that gives up, or a
// malformed command, sets the error flag; the warp then drains its copies
// and still takes every remaining barrier.
template <typename T>
__device__ __forceinline__ void refactor_body(const StreamDev& P, const SchedDev& S, const BatchDev& D,
                                              int BX, int NW) {
  using R = Rf<T>;
  const int g = BX;
  if (!D.gact[g]) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar[kMaxRefactorWarps][2];
  __shared__ int flags[2][32];
  __shared__ int prog[kMaxRefactorWarps];  // levels each warp has published (progress flags)
  __shared__ volatile int timed_out;
  constexpr uint32_t RB = R::RB;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = NW;
  const int CW = P.chunk_words;
  int32_t* cbuf = reinterpret_cast<int32_t*>(smem_raw) + (size_t)warp * 2 * CW;
  const uint32_t ring_s = smem_u32(smem_raw + (size_t)nw * 2 * CW * 4);
  const uint32_t ring_lane = ring_s + (uint32_t)lane * sizeof(T);
  const int s = g * 32 + lane;
  T* LUg = (T*)D.lu + (size_t)g * S.n_slots * 32u;
  T* Xg = (T*)D.sol + (size_t)g * S.n_u * 32u;
  const T* RHSg = (const T*)D.rhs + (size_t)g * S.n_u * 32u;
  const float ptol = D.piv_tol;
  const bool fuse = S.fuse_fwd != 0;
  bool bad = false, tiny = false;

  if (threadIdx.x < 64) (&flags[0][0])[threadIdx.x] = 0;
  if (threadIdx.x < kMaxRefactorWarps) prog[threadIdx.x] = 0;
  if (threadIdx.x == 0) timed_out = 0;
  if (lane == 0) {
    mbar_init(&mbar[warp][0]);
    mbar_init(&mbar[warp][1]);
  }
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  // the zero row (padding terms of the forward substitution read it)
  if (warp == 0) sts(ring_lane + (uint32_t)P.rows_total * RB, (T)0);
  __syncthreads();

  // warps beyond the plan's (a CTA sized for another topology's larger
  // plan, in a launch over several topologies) run no stream: they only
  // take the plan's barriers
  const bool runs = warp < nw;
  const int32_t* gw = runs ? P.words + (size_t)P.chunk0[warp] * CW : P.words;
  const int nch = runs ? P.nchunks[warp] : 0;
  if (runs && lane == 0) {
    bulk_load(cbuf, gw, (unsigned)CW * 4u, &mbar[warp][0]);
    if (nch > 1) bulk_load(cbuf + CW, gw + CW, (unsigned)CW * 4u, &mbar[warp][1]);
  }
  // bulk copies issued into / completions waited for, per chunk buffer (warp
  // uniform): a warp that stops early waits for the copies still in flight
  // before the CTA can exit
  int issued0 = runs ? 1 : 0, issued1 = nch > 1 ? 1 : 0, waited0 = 0, waited1 = 0;
  unsigned par0 = 0u, par1 = 0u;
  bool ok = runs && mbar_wait(&mbar[warp][0], par0);
  if (ok) waited0++;
  par0 ^= 1u;
  int chunk = 0, buf = 0, pc = 0, bars = 0, lev = 0;
  const int32_t* cb = cbuf;
  while (ok) {
    const int32_t w0 = cb[pc];
    const int op = w0 & 15;
    if (op == CMD_COLUMN) {
      const int k = cb[pc + 1], base = cb[pc + 2], ul = cb[pc + 3];
      const uint32_t h4 = (uint32_t)cb[pc + 4], h5 = (uint32_t)cb[pc + 5];
      const int nfw = cb[pc + 6];
      const uint32_t st_row = h4 & 0xffffu;
      const int nlate = (int)(h4 >> 16), npref = (int)(h5 & 0xffffu), nst = (int)(h5 >> 16);
      const int32_t* wl = cb + pc + 8;
      if (nlate) {
        R::gather(wl, nlate, ring_s, lane, LUg, Xg, RHSg, S.n_slots, S.n_u);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
      }
      if (npref) {
        R::gather(wl + nlate, npref, ring_s, lane, LUg, Xg, RHSg, S.n_slots, S.n_u);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
      }
      if ((w0 >> 7) & 1) {
        cp_async_wait_n((w0 >> 4) & 7);
        __syncwarp();
      }
      const int sw = (pc + 8 + nlate + npref + 3) & ~3;
      const uint32_t st_lane = ring_lane + st_row * RB;
      R::steps(reinterpret_cast<const uint4*>(cb + sw), nst, st_lane, ring_lane);
      const int ulen = ul & 0xffff, llen = (ul >> 16) & 0xffff;
      if (fuse)
        R::fwd(cb + sw + 4 * nst, nfw, cb[pc + 7], !((w0 >> 9) & 1),
               st_lane + (uint32_t)(ulen + 1 + llen) * RB, ring_lane);
      if (!((w0 >> 10) & 1)) R::finish(k, base, ulen, llen, st_lane, LUg, Xg, lane, fuse, ptol, bad, tiny);
      pc = sw + 4 * nst + nfw;
      if ((w0 >> 8) & 1) {
        if (P.sync) {
          publish_level(prog, warp, lane, ++lev);
        } else {
          __syncthreads();
          bars++;
        }
      }
    } else if (op == CMD_BWD) {
      const uint32_t w2 = (uint32_t)cb[pc + 2], w3 = (uint32_t)cb[pc + 3], w4 = (uint32_t)cb[pc + 4];
      const int k = cb[pc + 1];
      const int m = (int)(w3 >> 16), nlate = (int)(w4 & 0xffffu), npref = (int)(w4 >> 16);
      const int32_t* wl = cb + pc + 5;
      if (nlate) {
        R::gather(wl, nlate, ring_s, lane, LUg, Xg, RHSg, S.n_slots, S.n_u);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
      }
      if (npref) {
        R::gather(wl + nlate, npref, ring_s, lane, LUg, Xg, RHSg, S.n_slots, S.n_u);
        asm volatile("cp.async.commit_group;\n" ::: "memory");
      }
      if ((w0 >> 7) & 1) {
        cp_async_wait_n((w0 >> 4) & 7);
        __syncwarp();
      }
      R::bwd(wl + nlate + npref, m, (int)(((uint32_t)w0) >> 20), ring_lane + (w2 & 0xffffu) * RB,
             ring_lane + (w2 >> 16) * RB, ring_lane + (w3 & 0xffffu) * RB, ring_lane,
             Xg + (size_t)k * 32u + lane, bad);
      pc += 5 + nlate + npref + m;
      if ((w0 >> 8) & 1) {
        if (P.sync) {
          publish_level(prog, warp, lane, ++lev);
        } else {
          __syncthreads();
          bars++;
        }
      }
    } else {
      switch (op) {
        case CMD_STEPS: {
          const int m = (w0 >> 4) & 0xfff;
          const int first = (pc + 1 + 3) & ~3;
          R::steps(reinterpret_cast<const uint4*>(cb + first), m,
                   ring_lane + (((uint32_t)w0) >> 16) * RB, ring_lane);
          pc = first + 4 * m;
          break;
        }
        case CMD_GATHER: {
          const int m = (w0 >> 4) & 0xffff;
          R::gather(cb + pc + 1, m, ring_s, lane, LUg, Xg, RHSg, S.n_slots, S.n_u);
          if ((w0 >> 23) & 1) asm volatile("cp.async.commit_group;\n" ::: "memory");
          pc += 1 + m;
          break;
        }
        case CMD_WAIT:
          cp_async_wait_n((w0 >> 4) & 7);
          __syncwarp();
          pc++;
          break;
        case CMD_FWD: {
          const int m = (w0 >> 4) & 0xffff;
          const uint32_t w1 = (uint32_t)cb[pc + 1];
          R::fwd(cb + pc + 2, m, (int)(((uint32_t)w0) >> 21), (w0 >> 20) & 1,
                 ring_lane + ((w1 & 0xffffu) + (w1 >> 16)) * RB, ring_lane);
          pc += 2 + m;
          break;
        }
        case CMD_FINISH: {
          const int ulen = cb[pc + 3] & 0xffff, llen = (cb[pc + 3] >> 16) & 0xffff;
          R::finish(cb[pc + 1], cb[pc + 2], ulen, llen, ring_lane + (uint32_t)cb[pc + 4] * RB, LUg,
                    Xg, lane, fuse, ptol, bad, tiny);
          pc += 5;
          break;
        }
        case CMD_BAR:
          if (P.sync) {  // not in a plan with progress flags
            ok = false;
            break;
          }
          __syncthreads();
          bars++;
          pc++;
          break;
        case CMD_PUB:
          lev = (int)(((uint32_t)w0) >> 4);
          publish_level(prog, warp, lane, lev);
          pc++;
          break;
        case CMD_WAITP: {
          const int m = (w0 >> 4) & 0xff;
          if (!P.sync || pc + 1 + m >= CW || !wait_levels(cb + pc + 1, m, prog, &timed_out)) {
            ok = false;
            break;
          }
          __syncwarp();
          pc += 1 + m;
          break;
        }
        case CMD_NOP:
          pc++;
          break;
        case CMD_NEXT:
          __syncwarp();
          if (chunk + 2 < nch) {
            if (lane == 0)
              bulk_load(cbuf + (size_t)buf * CW, gw + (size_t)(chunk + 2) * CW, (unsigned)CW * 4u,
                        &mbar[warp][buf]);
            if (buf == 0) issued0++;
            else issued1++;
          }
          chunk++;
          buf ^= 1;
          if (chunk >= nch) {
            ok = false;
            break;
          }
          if (buf == 0) {
            ok = mbar_wait(&mbar[warp][0], par0);
            if (ok) waited0++;
            par0 ^= 1u;
          } else {
            ok = mbar_wait(&mbar[warp][1], par1);
            if (ok) waited1++;
            par1 ^= 1u;
          }
          cb = cbuf + (size_t)buf * CW;
          pc = 0;
          break;
        case CMD_END:
          goto done;
        default:
          ok = false;
      }
    }
    if (pc >= CW) ok = false;  // a command ran past its chunk
  }
done:
  if (!runs)
    for (; bars < P.n_bars; bars++) __syncthreads();
  if (!ok && runs) {
    if (lane == 0) atomicExch((int*)&timed_out, 1);
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    // stream chunks still being copied into this warp's buffers: wait for
    // them (each wait bounded) so no copy lands after the CTA has exited
    for (unsigned pr = (unsigned)waited0 & 1u; waited0 < issued0; waited0++, pr ^= 1u)
      if (!mbar_wait(&mbar[warp][0], pr)) break;
    for (unsigned pr = (unsigned)waited1 & 1u; waited1 < issued1; waited1++, pr ^= 1u)
      if (!mbar_wait(&mbar[warp][1], pr)) break;
    for (; bars < P.n_bars; bars++) __syncthreads();
  }
  if (bad) atomicOr(&flags[0][lane], 1);
  if (tiny) atomicOr(&flags[1][lane], 1);
  __syncthreads();
  if (warp == 0) {
    if (flags[0][lane]) D.sing[s] = 1;
    if (flags[1][lane]) D.piv_flag[s] = 1;
    if (lane == 0 && timed_out && D.err) atomicExch(D.err, 1);
  }
  // every copy into this warp's chunk buffers has completed (waited for, or
  // drained on an error): the barriers may be initialized again by the next
  // refactor a persistent CTA runs
  if (lane == 0) {
    mbar_inval(&mbar[warp][0]);
    mbar_inval(&mbar[warp][1]);
  }
}
template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 32 * kMaxRefactorWarps : 256, 1)
    k_refactor(StreamDev P, SchedDev S, BatchDev D) {
  refactor_body<T>(P, S, D, blockIdx.x, blockDim.x >> 5);
}

// ---------------------------------------------------------------------------
// K3 / K4 wide levels.  The first levels of the refactor hold most columns
// (case2000: 2,900 of 3,698 in levels 0-9), all independent within a level;
// the last phases of the backward substitution likewise hold most rows.
// The wide kernels run one such level / phase per launch with one warp per
// (column or row, group of 32 scenarios), so a level's work spreads over
// every SM whatever the batch size, where the per-group stream kernel would
// give it one SM per group.  A column's values are staged in shared memory
// private to its warp's lanes (row r of lane l at stage[r * 32 + l], `rows`
// rows per warp: the plan's longest wide column); its
// inputs -- the A image the fill wrote into the factor, the L values and y
// of earlier columns -- come from global memory, where earlier launches
// left them.  The arithmetic is the stream kernel's, in the same order per
// value: KLU's update order (the schedule's hazard-free batches keep each
// entry's order), the forward terms in order, the pivot's correctly
// rounded reciprocal, the pivot-ratio check; so both give the same bits.
constexpr int kWideWarps = 4;  // warps per CTA of the wide kernels

template <typename T>
__device__ __forceinline__ void refactor_wide_body(const SchedDev& S, const BatchDev& D, int lev,
                                                   int groups, int BX, int rows) {
  extern __shared__ __align__(16) unsigned char wsm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int q0 = S.lev_ptr[lev], ncol = S.lev_ptr[lev + 1] - q0;
  const long long task = (long long)BX * kWideWarps + warp;
  if (task >= (long long)ncol * groups) return;
  const int g = (int)(task % groups), q = (int)(task / groups);
  if (!D.gact[g]) return;
  T* stg = reinterpret_cast<T*>(wsm) + (size_t)warp * rows * 32 + lane;
  const int k = S.lev_cols[q0 + q];
  const int base = S.c_base[k], ulen = S.c_ulen[k], len = ulen + 1 + S.c_llen[k];
  const T* LUr = (const T*)D.lu + (size_t)g * S.n_slots * 32u + lane;
  T* LUw = (T*)D.lu + (size_t)g * S.n_slots * 32u + lane;
  for (int r = 0; r < len; r++) stg[r * 32] = LUr[(size_t)(base + r) * 32];
  // updates: per hazard-free batch, every load before every store
  int o = S.op_ptr[k];
  for (int b = S.bt_ptr[k]; b < S.bt_ptr[k + 1]; b++) {
    const int cnt = S.bt_cnt[b];
    T lv[kMaxBatch], uv[kMaxBatch], dv[kMaxBatch];
    int dp[kMaxBatch];
#pragma unroll
    for (int t = 0; t < kMaxBatch; t++)
      if (t < cnt) {
        const uint32_t pos = S.op_pos[o + t];
        dp[t] = (int)(pos & 0xffffu);
        lv[t] = LUr[(size_t)S.op_slot[o + t] * 32];
        uv[t] = stg[(pos >> 16) * 32];
        dv[t] = stg[dp[t] * 32];
      }
#pragma unroll
    for (int t = 0; t < kMaxBatch; t++)
      if (t < cnt) stg[dp[t] * 32] = dv[t] - lv[t] * uv[t];
    o += cnt;
  }
  T* Xg = (T*)D.sol + (size_t)g * S.n_u * 32u + lane;
  T y = (T)0;
  if (S.fuse_fwd) {
    y = ((const T*)D.rhs)[((size_t)g * S.n_u + k) * 32u + lane];
    for (int tt = S.fw_ptr[k]; tt < S.fw_ptr[k + 1]; tt++)
      y -= LUr[(size_t)S.fw_slot[tt] * 32] * Xg[(size_t)S.fw_col[tt] * 32];
  }
  // finish: pivot, U and the diagonal as they are, L scaled
  const T piv = stg[ulen * 32];
  const bool bad = piv == (T)0;
  const T inv = rcp_rn(piv);
  for (int r = 0; r <= ulen; r++) LUw[(size_t)(base + r) * 32] = stg[r * 32];
  T colmax = fabs(piv);
  for (int r = ulen + 1; r < len; r++) {
    T v = stg[r * 32];
    colmax = fmax(colmax, fabs(v));
    v *= inv;
    LUw[(size_t)(base + r) * 32] = v;
  }
  const float ptol = D.piv_tol;
  const bool tiny = (ptol > 0.0f) && ((float)fabs(piv) < ptol * (float)colmax);
  if (S.fuse_fwd) Xg[(size_t)k * 32] = y;
  const int s = g * 32 + lane;
  if (bad) D.sing[s] = 1;
  if (tiny) D.piv_flag[s] = 1;
}
template <typename T>
__global__ void __launch_bounds__(32 * kWideWarps) k_refactor_wide(SchedDev S, BatchDev D, int lev,
                                                                   int groups, int rows) {
  refactor_wide_body<T>(S, D, lev, groups, blockIdx.x, rows);
}

// The backward substitution of one wide refactor level's rows: x_k = (y_k -
// sum U(k, j) x_j) / U(k, k), terms in the stream's order, one warp per
// (row, group).  A row needs only rows of higher levels, so the levels run
// from the last wide one down, after the stream kernel has solved the rest.
template <typename T>
__device__ __forceinline__ void solve_wide_body(const SchedDev& S, const BatchDev& D, int lev,
                                                int groups, int BX) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int q0 = S.lev_ptr[lev], nrow = S.lev_ptr[lev + 1] - q0;
  const long long task = (long long)BX * kWideWarps + warp;
  if (task >= (long long)nrow * groups) return;
  const int g = (int)(task % groups), q = (int)(task / groups);
  if (!D.gact[g]) return;
  const int k = S.lev_cols[q0 + q];
  const T* LUr = (const T*)D.lu + (size_t)g * S.n_slots * 32u + lane;
  T* Xg = (T*)D.sol + (size_t)g * S.n_u * 32u + lane;
  T v = Xg[(size_t)k * 32];
  for (int tt = S.bw_ptr[k]; tt < S.bw_ptr[k + 1]; tt++)
    v -= LUr[(size_t)S.bw_slot[tt] * 32] * Xg[(size_t)S.bw_col[tt] * 32];
  const T x = v / LUr[(size_t)S.diag_slot[k] * 32];
  if (!isfinite(x)) D.sing[g * 32 + lane] = 1;
  Xg[(size_t)k * 32] = x;
}
template <typename T>
__global__ void __launch_bounds__(32 * kWideWarps) k_solve_wide(SchedDev S, BatchDev D, int lev,
                                                                int groups) {
  solve_wide_body<T>(S, D, lev, groups, blockIdx.x);
}

// ---------------------------------------------------------------------------
// Many topologies in one launch per phase.  A job is one topology's batch:
// its schedule, batch buffers and refactor stream.  A launch covers a list
// of jobs: off[k] .. off[k+1] are the CTAs of the list's k-th job (its
// blocks of every group, group-major), so a CTA finds its job by binary
// search over the n + 1 offsets, copies the job's descriptors into shared
// memory and runs the same body as the single-topology kernel on them:
// every scenario's arithmetic is the same.  The refactor's list names the
// largest jobs first, so the block scheduler starts the longest dependency
// chains first.
struct __align__(16) MultiJob {
  SchedDev S;
  BatchDev D;
  StreamDev P;
  int nw;  // warps of the job's refactor plan
};
static_assert(sizeof(MultiJob) % 16 == 0, "jobs are copied as int4");

struct MultiList {
  const int32_t* off;  // [n + 1] first CTA of each listed job
  const int32_t* job;  // [n] job index
  int n;
};

// the listed job of this CTA (its copy in J) and the CTA's index within it
__device__ __forceinline__ int enter_job(MultiJob& J, const MultiJob* __restrict__ jobs,
                                         const MultiList& L) {
  const int b = blockIdx.x;
  int lo = 0, hi = L.n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (L.off[mid] <= b) lo = mid;
    else hi = mid;
  }
  const int4* a = reinterpret_cast<const int4*>(jobs + L.job[lo]);
  int4* d = reinterpret_cast<int4*>(&J);
  for (int i = threadIdx.x; i < (int)(sizeof(MultiJob) / 16); i += blockDim.x) d[i] = a[i];
  __syncthreads();
  return b - L.off[lo];
}

// CTAs per group of each kernel (the single-topology grids' x extent)
__device__ __host__ __forceinline__ int update_blocks(int n_bus) { return (n_bus + 7) / 8; }
__device__ __host__ __forceinline__ int inject_blocks(int n_bus) { return (n_bus + 31) / 32; }
__device__ __host__ __forceinline__ int fill_blocks(int n_ftask, int n_fzero) {
  return ((n_ftask + 7) / 8 + (n_fzero + 31) / 32 + 7) / 8;
}

template <typename T>
__global__ void __launch_bounds__(256) k_update_multi(const MultiJob* __restrict__ jobs,
                                                      MultiList L, int it, int mode) {
  __shared__ __align__(16) MultiJob J;
  const int b = enter_job(J, jobs, L), nb = update_blocks(J.S.n_bus);
  update_body<T>(J.S, J.D, it, mode, b % nb, b / nb);
}
template <typename T>
__global__ void __launch_bounds__(256) k_inject_multi(const MultiJob* __restrict__ jobs,
                                                      MultiList L, int it) {
  __shared__ __align__(16) MultiJob J;
  const int b = enter_job(J, jobs, L), nb = inject_blocks(J.S.n_bus);
  inject_body<T, false, 4, false>(J.S, J.D, it, b % nb, b / nb);
}
__global__ void k_decide_multi(const MultiJob* __restrict__ jobs, MultiList L, int it, int mode) {
  __shared__ __align__(16) MultiJob J;
  const int b = enter_job(J, jobs, L);
  decide_body(J.D, it, mode, b);
}
template <typename T>
__global__ void __launch_bounds__(256) k_fill_multi(const MultiJob* __restrict__ jobs, MultiList L) {
  __shared__ __align__(16) MultiJob J;
  const int b = enter_job(J, jobs, L), nb = fill_blocks(J.S.n_ftask, J.S.n_fzero);
  fill_body<T, false>(J.S, J.D, (J.S.n_ftask + 7) / 8, 8, b % nb, b / nb);
}
template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 4 ? 32 * kMaxRefactorWarps : 256, 1)
    k_refactor_multi(const MultiJob* __restrict__ jobs, MultiList L) {
  __shared__ __align__(16) MultiJob J;
  const int b = enter_job(J, jobs, L);
  refactor_body<T>(J.P, J.S, J.D, b, J.nw);
}
// one wide level `lev` of every listed job (each job's CTAs: its columns of
// that level times its groups, kWideWarps tasks per CTA)
template <typename T>
__global__ void __launch_bounds__(32 * kWideWarps) k_refactor_wide_multi(
    const MultiJob* __restrict__ jobs, MultiList L, int lev, int rows) {
  __shared__ __align__(16) MultiJob J;
  const int b = enter_job(J, jobs, L);
  refactor_wide_body<T>(J.S, J.D, lev, J.D.G, b, rows);
}
template <typename T>
__global__ void __launch_bounds__(32 * kWideWarps) k_solve_wide_multi(
    const MultiJob* __restrict__ jobs, MultiList L, int lev) {
  __shared__ __align__(16) MultiJob J;
  const int b = enter_job(J, jobs, L);
  solve_wide_body<T>(J.S, J.D, lev, J.D.G, b);
}
// ---------------------------------------------------------------------------
// The persistent many-topology Newton kernel.  Each CTA (one per SM, as
// many warps as the largest refactor plan; the mismatch and fill phases use
// its first 8, the kernels' block) takes work items {job, group} from a device-side queue (listed largest
// job first) and runs that group's whole Newton loop: update, injections,
// decision, fill and refactor, one after the other with CTA barriers between
// them, until its scenarios have converged or failed, then takes the next
// item.  The phases are the single-topology kernels' bodies with the same
// block coordinates (a loop over the blocks a group has in each kernel), so
// every scenario's arithmetic is that of its single solve; a group that
// leaves early skips only iterations that would leave its values unchanged
// (no lane running: the update moves nothing, the rotation by a zero step
// returns the same cos / sin).
// the CTA: as wide as the largest plan it runs (FP32 up to 12 warps, FP64 8)
template <typename T>
constexpr int persist_threads() { return sizeof(T) == 4 ? 32 * kMaxRefactorWarps : 256; }
template <typename T>
__device__ __forceinline__ void newton_group(const MultiJob& J, int g, int max_iter) {
  const SchedDev& S = J.S;
  const BatchDev& D = J.D;
  const int nbu = update_blocks(S.n_bus), nbi = inject_blocks(S.n_bus);
  const int nbf = fill_blocks(S.n_ftask, S.n_fzero), tw = (S.n_ftask + 7) / 8;
  int it = 0;
  for (; it < max_iter; it++) {
    for (int b = 0; b < nbu; b++) update_body<T>(S, D, it, 0, b, g);
    __syncthreads();
    for (int b = 0; b < nbi; b++) {
      inject_body<T, false, 4, false>(S, D, it, b, g);
      __syncthreads();  // its block reduction's shared row is reused by the next block
    }
    if (threadIdx.x < 32) decide_body(D, it, 0, g);
    __syncthreads();
    if (!D.gact[g]) break;
    for (int b = 0; b < nbf; b++) fill_body<T, false>(S, D, tw, 8, b, g);
    __syncthreads();
    refactor_body<T>(J.P, S, D, g, J.nw);
    __syncthreads();
  }
  if (it == max_iter) {
    // the budget ran out with lanes running: their MaxIterations step
    for (int b = 0; b < nbu; b++) update_body<T>(S, D, max_iter, 1, b, g);
    __syncthreads();
    if (threadIdx.x < 32) decide_body(D, max_iter, 1, g);
    __syncthreads();
  }
}
template <typename T>
__global__ void __launch_bounds__(persist_threads<T>(), 1)
    k_newton_persistent(const MultiJob* __restrict__ jobs, const int2* __restrict__ items,
                        int n_items, int* __restrict__ next, int max_iter) {
  __shared__ __align__(16) MultiJob J;
  __shared__ int item;
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(next, 1);
    __syncthreads();
    const int q = item;
    if (q >= n_items) return;
    const int2 w = items[q];
    const int4* a = reinterpret_cast<const int4*>(jobs + w.x);
    int4* d = reinterpret_cast<int4*>(&J);
    for (int i = threadIdx.x; i < (int)(sizeof(MultiJob) / 16); i += blockDim.x) d[i] = a[i];
    __syncthreads();
    newton_group<T>(J, w.y, max_iter);
    __syncthreads();  // every thread is done with J and `item` before the next item
  }
}

// every job's running-group counter to zero / into one array (one read back)
__global__ void k_multi_counts(const MultiJob* __restrict__ jobs, int n, int32_t* out, int zero) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    if (zero) *jobs[j].D.nactive = 0;
    else out[j] = *jobs[j].D.nactive;
  }
}

// ---------------------------------------------------------------------------
// Linear initial guess (src/network.rs:627-678).  The PQ buses' voltages U_n
// solve Y'_nn U_n = -Y'_ns U_s, where Y' is the Y-bus with -conj(S_i) added
// on the diagonal of each PQ bus i (its injection as a constant admittance
// at |V| = 1) and U_s the fixed voltages of the other buses.  The complex
// system is solved as the real one with the block [[Re, -Im], [Im, Re]] per
// entry (unknowns Re U_r, Im U_r at 2r, 2r + 1), refactored in FP64 with the
// pivot order of its first factorization.
struct GuessDev {
  int n_bus, m, n2, n_slots, n_off;
  const int32_t *yp, *yi;
  const double *yre, *yim;
  // per LU slot, then per off-diagonal entry: {part (-1: zero fill-in, 0: Re,
  // 1: -Im, 2: Im), Y entry (-1: none), PQ bus of the load term (-1: none), 0}
  const int4* rec;
  const int32_t* rhs_ptr;  // [m + 1]: per PQ row, its neighbours of fixed voltage
  const int2* rhs_ej;      // {Y entry, bus}
  const int32_t* pq_bus;   // [m]
  const int32_t* pinv;     // [n2]: factor row of real equation q
  const int32_t* qinv;     // [n2]: factor column of real unknown u
  const double* zip;       // ZIP terms as in SchedDev, or null
};

// Y entry e of scenario s, with its outage delta (the scenario's four Y slots)
__device__ __forceinline__ void guess_y(const GuessDev& L, int e, const int32_t* os, const double* odr,
                                        const double* odi, double& yr, double& yi) {
  yr = e >= 0 ? L.yre[e] : 0.0;
  yi = e >= 0 ? L.yim[e] : 0.0;
  if (os && e >= 0)
    for (int c = 0; c < 4; c++)
      if (os[c] == e) {
        yr += odr[c];
        yi += odi[c];
      }
}

// Values of the guess system in its factor's layout and its right-hand side
// in pivot order, per scenario (lane).  grid (ceil(items / 8), G): a warp per
// item, the LU slots and off-diagonal entries, then the PQ rows.
__global__ void __launch_bounds__(256) k_guess_fill(GuessDev L, int B, const double* __restrict__ p,
                                                     const double* __restrict__ q,
                                                     const double* __restrict__ vm0,
                                                     const double* __restrict__ va0, int v_stride,
                                                     const int32_t* __restrict__ o_slot,
                                                     const double* __restrict__ o_dre,
                                                     const double* __restrict__ o_dim, double* lu,
                                                     double* off, double* rhs) {
  const int g = blockIdx.y, lane = threadIdx.x & 31;
  const int item = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int s = min(g * 32 + lane, B - 1);
  const int N = L.n_bus;
  const int32_t* os = o_slot ? o_slot + 4 * s : nullptr;
  const double* odr = o_slot ? o_dre + 4 * s : nullptr;
  const double* odi = o_slot ? o_dim + 4 * s : nullptr;
  if (os && os[0] < 0) os = nullptr;
  const int nv = L.n_slots + L.n_off;
  if (item < nv) {
    const int4 r = __ldg(L.rec + item);
    double v = 0.0;
    if (r.x >= 0) {
      double yr, yi;
      guess_y(L, r.y, os, odr, odi, yr, yi);
      if (r.z >= 0) {  // + (-conj(p + jq)) = -p + jq, the effective injection at the start |V|
        const double v = vm0[(size_t)s * v_stride + r.z];
        yr -= eff_inj(L.zip, N, r.z, 0, p[(size_t)s * N + r.z], v);
        yi += eff_inj(L.zip, N, r.z, 1, q[(size_t)s * N + r.z], v);
      }
      v = r.x == 0 ? yr : (r.x == 1 ? -yi : yi);
    }
    if (item < L.n_slots) lu[((size_t)g * L.n_slots + item) * 32 + lane] = v;
    else off[((size_t)g * L.n_off + (item - L.n_slots)) * 32 + lane] = v;
    return;
  }
  const int r = item - nv;
  if (r >= L.m) return;
  double ar = 0.0, ai = 0.0;  // sum of Y_ij U_j over the fixed neighbours
  for (int t = __ldg(L.rhs_ptr + r); t < __ldg(L.rhs_ptr + r + 1); t++) {
    const int2 ej = __ldg(L.rhs_ej + t);
    double yr, yi;
    guess_y(L, ej.x, os, odr, odi, yr, yi);
    const size_t xv = (size_t)s * v_stride + ej.y;
    double sn, cs;
    sincos(va0[xv], &sn, &cs);
    const double ur = vm0[xv] * cs, ui = vm0[xv] * sn;
    ar += yr * ur - yi * ui;
    ai += yr * ui + yi * ur;
  }
  rhs[((size_t)g * L.n2 + __ldg(L.pinv + 2 * r)) * 32 + lane] = -ar;
  rhs[((size_t)g * L.n2 + __ldg(L.pinv + 2 * r + 1)) * 32 + lane] = -ai;
}

// The start point: every bus's given voltage, then the PQ buses' solution
// where the scenario's guess system was regular and the solution finite
// (else they keep the given one, as the reference does when its solve fails).
// (grid-stride loops: the launch's grid is capped)
__global__ void k_guess_start(int B, int N, const double* __restrict__ vm0,
                              const double* __restrict__ va0, int v_stride, double* gvm, double* gva) {
  const size_t total = (size_t)B * N;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t s = i / N, b = i % N;
    gvm[i] = vm0[s * v_stride + b];
    gva[i] = va0[s * v_stride + b];
  }
}
__global__ void k_guess_out(GuessDev L, int B, const double* __restrict__ sol,
                            const int32_t* __restrict__ sing, double* gvm, double* gva) {
  const size_t total = (size_t)B * L.m;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(i / L.m), r = (int)(i % L.m);
    const int g = s / 32, lane = s % 32;
    const double re = sol[((size_t)g * L.n2 + __ldg(L.qinv + 2 * r)) * 32 + lane];
    const double im = sol[((size_t)g * L.n2 + __ldg(L.qinv + 2 * r + 1)) * 32 + lane];
    if (sing[s] != 0 || !isfinite(re) || !isfinite(im)) continue;
    const size_t x = (size_t)s * L.n_bus + __ldg(L.pq_bus + r);
    gvm[x] = hypot(re, im);
    gva[x] = atan2(im, re);
  }
}

// ---------------------------------------------------------------------------
// K4: substitution phases (dependency levels), one CTA per group.  Forward
// phases (kind 0) fold the off-diagonal terms of later BTF blocks into the
// right-hand side; backward phases (kind 1) divide by U(k,k).
template <typename T>
__global__ void __launch_bounds__(256) k_solve(SchedDev S, BatchDev D) {
  constexpr int CH = 4;
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
      const int* tslot = kind == 0 ? S.fw_slot : S.bw_slot;
      const int* tcol = kind == 0 ? S.fw_col : S.bw_col;
      const int tb = __ldg((kind == 0 ? S.fw_ptr : S.bw_ptr) + k);
      const int te = __ldg((kind == 0 ? S.fw_ptr : S.bw_ptr) + k + 1);
      T d = (T)1;
      if (kind == 1) d = LU[luG + (size_t)__ldg(S.diag_slot + k) * 32u + lane];
      T v = kind == 0 ? RHS[xG + (size_t)k * 32u + lane] : X[xG + (size_t)k * 32u + lane];
      for (int t0 = tb; t0 < te; t0 += CH) {
        T c[CH], xv[CH];
#pragma unroll
        for (int t = 0; t < CH; t++)
          if (t0 + t < te) {
            const int sl = __ldg(tslot + t0 + t);
            c[t] = (sl >= 0) ? LU[luG + (size_t)sl * 32u + lane] : OFF[gidx(g, S.n_off, -sl - 1, lane)];
            xv[t] = X[xG + (size_t)__ldg(tcol + t0 + t) * 32u + lane];
          }
#pragma unroll
        for (int t = 0; t < CH; t++)
          if (t0 + t < te) v -= c[t] * xv[t];
      }
      if (kind == 1) {
        v = v / d;
        if (!isfinite((double)v)) bad = true;
      }
      X[xG + (size_t)k * 32u + lane] = v;
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
