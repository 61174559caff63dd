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
  unsigned long long* maxacc;      // max |F| of the running iteration (bits of a double >= 0)
  double *hist;                    // [G*32][max_iter] or null
  int32_t *gact;                   // [G] group has a running lane
  int32_t *nactive;                // [1] running groups after the last decision
  // optional per-scenario outage: 4 Y slots + deltas, and the branch buses
  const int32_t *o_slot, *o_bf, *o_bt;
  const double *o_dre, *o_dim;
  float piv_tol;                   // pivot-ratio threshold (mixed path)
  int32_t* err;                    // [0] set when a bounded device wait gave up
};

__device__ __forceinline__ size_t gidx(int g, int n, int e, int lane) {
  return ((size_t)g * (size_t)n + (size_t)e) * 32u + (size_t)lane;
}

// ---------------------------------------------------------------------------
// K5 + K1a.  grid (ceil(N/8), G), 8 warps: warp -> bus, lane -> scenario.
// mode 0: iteration `it`; mode 1: the update after the last iteration.
template <typename T>
__global__ void __launch_bounds__(256) k_update(SchedDev S, BatchDev D, int it, int mode) {
  const int g = blockIdx.y;
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int N = S.n_bus;
  if (i >= N) return;
  const int s = g * 32 + lane;
  const bool upd = D.status[s] == ST_RUNNING && (it > 0 || mode == 1) && D.sing[s] == 0;
  const size_t x = gidx(g, N, i, lane);
  double vm = D.vm[x], va = D.va[x];
  if (upd) {
    const T* sol = (const T*)D.sol;
    const int ca = __ldg(S.bus_colA + i), cv = __ldg(S.bus_colV + i);
    if (ca >= 0) va += (double)sol[gidx(g, S.n_u, ca, lane)];
    if (cv >= 0) vm += (double)sol[gidx(g, S.n_u, cv, lane)];
    D.vm[x] = vm;
    D.va[x] = va;
  }
  if (mode != 0) return;
  double sn, cs;
  sincos(va, &sn, &cs);
  const double e = vm * cs, f = vm * sn;
  D.e[x] = e;
  D.f[x] = f;
  ((T*)D.eT)[x] = (T)e;
  ((T*)D.fT)[x] = (T)f;
  ((T*)D.ivT)[x] = (T)(1.0 / vm);
}

// ---------------------------------------------------------------------------
// K1b: S = V conj(Y V), F, max|F|.  grid (ceil(N / (8*BPW)), G), 8 warps,
// each warp BPW consecutive buses; neighbour loads issued 8 at a time.
template <typename T, bool OUTAGE, int BPW>
__global__ void __launch_bounds__(256) k_inject(SchedDev S, BatchDev D, int it) {
  const int g = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int s = g * 32 + lane;
  const int N = S.n_bus;
  __shared__ double red[8][32];
  const bool active = D.status[s] == ST_RUNNING && !(it > 0 && D.sing[s] != 0);
  T* rhs = (T*)D.rhs;
  int obf = -1, obt = -1;
  if (OUTAGE) { obf = D.o_bf[s]; obt = D.o_bt[s]; }
  double mx = 0.0;
  const int i0 = (blockIdx.x * 8 + warp) * BPW;
  for (int i = i0; i < min(N, i0 + BPW); i++) {
    double ir = 0.0, ii = 0.0;
    const int pb = __ldg(S.yp + i), pe = __ldg(S.yp + i + 1);
    for (int p = pb; p < pe; p += 8) {
      double ek[8], fk[8], gr[8], gi[8];
#pragma unroll
      for (int t = 0; t < 8; t++) {
        if (p + t < pe) {
          const int k = __ldg(S.yi + p + t);
          gr[t] = __ldg(S.yre + p + t);
          gi[t] = __ldg(S.yim + p + t);
          const size_t xk = gidx(g, N, k, lane);
          ek[t] = D.e[xk];
          fk[t] = D.f[xk];
        }
      }
#pragma unroll
      for (int t = 0; t < 8; t++) {
        if (p + t < pe) {
          ir += gr[t] * ek[t] - gi[t] * fk[t];
          ii += gr[t] * fk[t] + gi[t] * ek[t];
        }
      }
    }
    const size_t x = gidx(g, N, i, lane);
    const double ei = D.e[x], fi = D.f[x];
    if (OUTAGE && (i == obf || i == obt)) {
      const size_t xf = gidx(g, N, obf, lane), xt = gidx(g, N, obt, lane);
      const double ef = D.e[xf], ff = D.f[xf], et = D.e[xt], ft = D.f[xt];
      const int c0 = (i == obf) ? 0 : 2;
      const double ar = D.o_dre[4 * s + c0], ai = D.o_dim[4 * s + c0];
      const double br = D.o_dre[4 * s + c0 + 1], bi = D.o_dim[4 * s + c0 + 1];
      ir += ar * ef - ai * ff + br * et - bi * ft;
      ii += ar * ff + ai * ef + br * ft + bi * et;
    }
    const double pc = ei * ir + fi * ii;
    const double qc = fi * ir - ei * ii;
    const int rp = __ldg(S.bus_rowP + i), rq = __ldg(S.bus_rowQ + i);
    if (active) {
      if (rp >= 0) {
        const double F = D.psp[x] - pc;
        mx = fmax(mx, fabs(F));
        rhs[gidx(g, S.n_u, rp, lane)] = (T)F;
      }
      if (rq >= 0) {
        const double F = D.qsp[x] - qc;
        mx = fmax(mx, fabs(F));
        rhs[gidx(g, S.n_u, rq, lane)] = (T)F;
      }
    }
    ((T*)D.pT)[x] = (T)pc;
    ((T*)D.qT)[x] = (T)qc;
  }
  red[warp][lane] = mx;
  __syncthreads();
  if (warp == 0) {
    double m = 0.0;
#pragma unroll
    for (int w = 0; w < 8; w++) m = fmax(m, red[w][lane]);
    if (active && m > 0.0) atomicMax(D.maxacc + s, (unsigned long long)__double_as_longlong(m));
  }
}

// ---------------------------------------------------------------------------
// K1c: convergence decision (newton_raphson_cached's strict max|F| < tol,
// src/solver.rs:699-703).  grid G, one warp.
__global__ void k_decide(BatchDev D, int it, int mode) {
  const int g = blockIdx.x, lane = threadIdx.x;
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

// ---------------------------------------------------------------------------
// K2: Jacobian fill (src/jacobian.rs:202-250 formulas in rectangular form:
// V_i V_k cos(th_i - th_k) = e_i e_k + f_i f_k, V_i V_k sin(..) = f_i e_k - e_i f_k),
// written straight into the factor's layout: each LU slot receives its
// A entry or zero (fill-in), so the refactor starts a column with one bulk
// copy.  Index space: the LU slots, then the off-diagonal (BTF) entries.
// grid (chunks, G); each warp fills a contiguous run of slots.
template <typename T, bool OUTAGE>
__global__ void __launch_bounds__(256) k_fill(SchedDev S, BatchDev D, int per_warp) {
  const int g = blockIdx.y;
  if (!D.gact[g]) return;
  const int lane = threadIdx.x & 31;
  const int wglob = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int total = S.n_slots + S.n_off_real;
  const int a0 = wglob * per_warp;
  if (a0 >= total) return;
  const int a1 = min(total, a0 + per_warp);
  const int N = S.n_bus;
  const int s = g * 32 + lane;
  const T* eT = (const T*)D.eT; const T* fT = (const T*)D.fT; const T* ivT = (const T*)D.ivT;
  const T* pT = (const T*)D.pT; const T* qT = (const T*)D.qT;
  T* LU = (T*)D.lu;
  T* OFF = (T*)D.off;
  int os0 = -1, os1 = -1, os2 = -1, os3 = -1;
  if (OUTAGE && D.o_bf[s] >= 0) {
    os0 = D.o_slot[4 * s]; os1 = D.o_slot[4 * s + 1]; os2 = D.o_slot[4 * s + 2]; os3 = D.o_slot[4 * s + 3];
  }
  for (int x = a0; x < a1; x++) {
    const int a = (x < S.n_slots) ? __ldg(S.slot_a + x) : __ldg(S.off_a + (x - S.n_slots));
    T v = (T)0;
    if (a >= 0) {
      const int kind = __ldg(S.a_kind + a), i = __ldg(S.a_bi + a), k = __ldg(S.a_bk + a);
      const int ys = __ldg(S.a_yslot + a);
      double gd = __ldg(S.yre + ys), bd = __ldg(S.yim + ys);
      if (OUTAGE) {
        const int c = (ys == os0) ? 0 : (ys == os1) ? 1 : (ys == os2) ? 2 : (ys == os3) ? 3 : -1;
        if (c >= 0) { gd += D.o_dre[4 * s + c]; bd += D.o_dim[4 * s + c]; }
      }
      const T G = (T)gd, B = (T)bd;
      const size_t xi = gidx(g, N, i, lane);
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
    }
    if (x < S.n_slots) LU[gidx(g, S.n_slots, x, lane)] = v;
    else OFF[gidx(g, S.n_off, x - S.n_slots, lane)] = v;
  }
}

// Per-lane asynchronous copies global -> shared (cp.async, 4 or 8 bytes).
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit_wait() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}
template <typename T>
__device__ __forceinline__ void cp_async_t(T* smem, const T* gmem) {
  if (sizeof(T) == 8) cp_async8(smem, gmem); else cp_async4(smem, gmem);
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

// The next column (index into lev_cols) this warp takes after column q,
// or -1: columns of a level are dealt round-robin to the warps.
__device__ __forceinline__ int next_task(const SchedDev& S, int lv, int q, int warp, int nw) {
  if (q + nw < __ldg(S.lev_ptr + lv + 1)) return q + nw;
  for (int l = lv + 1; l < S.n_levels; l++) {
    const int c = __ldg(S.lev_ptr + l) + warp;
    if (c < __ldg(S.lev_ptr + l + 1)) return c;
  }
  return -1;
}

// One batch of N independent updates on the stage: all loads, then the
// FMAs, then the stores (no op of a batch touches an entry another writes).
template <typename T, int N>
__device__ __forceinline__ void run_batch(T* stl, const T* opvl, const int32_t* desc) {
  int dd[N];
  T xd[N], xu[N], lv[N];
#pragma unroll
  for (int t = 0; t < N; t++) {
    const uint32_t ps = (uint32_t)desc[2 * t + 1];
    dd[t] = (int)(ps & 0xffffu);
    xd[t] = stl[dd[t]];
    xu[t] = stl[ps >> 16];
    lv[t] = opvl[t * 32];
  }
#pragma unroll
  for (int t = 0; t < N; t++) stl[dd[t]] = xd[t] - lv[t] * xu[t];
}

// K3: refactor.  One CTA per group of 32 scenarios; the columns of each
// dependency level are dealt round-robin to the warps; __syncthreads
// between levels.  Per warp, in shared memory:
//   pkt[2][pkcap]  its current and next column packet (TMA bulk copies)
//   stage[cap][32] the column: [U (topological order) | diagonal | L],
//                  initialised by one TMA bulk copy of the A values and
//                  zeros the fill kernel left in the factor's layout
//   opv[opcap][32] the L(i, j) values its updates read (cp.async)
//   opd[opcap][2]  their descriptors when the packet could not hold them
//   dat[dcap][32]  forward-substitution terms and b_k
// Updates run as hazard-free batches dispatched to exact-size code.  With
// S.fuse_fwd the forward substitution y_k = b_k - sum_j L(k, j) y_j runs in
// the same sweep.
template <typename T>
__global__ void __launch_bounds__(256) k_refactor(SchedDev S, BatchDev D, int cap, int opcap,
                                                  int pkcap, int dcap) {
  const int g = blockIdx.x;
  if (!D.gact[g]) return;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t mbar[8][3];
  __shared__ int flags[2][32];
  __shared__ int timed_out;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const size_t wbytes = (size_t)2 * pkcap * 4 + (size_t)opcap * 8 +
                        ((size_t)cap + (size_t)opcap + (size_t)dcap) * 32 * sizeof(T);
  unsigned char* wbase = smem_raw + (size_t)warp * ((wbytes + 127) & ~(size_t)127);
  int32_t* pkb = reinterpret_cast<int32_t*>(wbase);
  int32_t* opd = pkb + (size_t)2 * pkcap;
  T* stage_w = reinterpret_cast<T*>(wbase + (size_t)2 * pkcap * 4 + (size_t)opcap * 8);
  T* opv = stage_w + (size_t)cap * 32;
  T* dat = opv + (size_t)opcap * 32;
  const int s = g * 32 + lane;
  T* LU = (T*)D.lu;
  T* X = (T*)D.sol;
  const T* RHS = (const T*)D.rhs;
  const size_t luG = (size_t)g * S.n_slots * 32u;
  const size_t xG = (size_t)g * S.n_u * 32u;
  T* LUg = LU + luG;
  bool bad = false, tiny = false;
  const float ptol = D.piv_tol;

  if (threadIdx.x < 64) (&flags[0][0])[threadIdx.x] = 0;
  if (threadIdx.x == 0) timed_out = 0;
  if (lane == 0) {
    mbar_init(&mbar[warp][0]);
    mbar_init(&mbar[warp][1]);
    mbar_init(&mbar[warp][2]);
  }
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  __syncthreads();

  auto issue = [&](int q, int buf) {
    const int off = __ldg(S.pk_off + q), sz = __ldg(S.pk_off + q + 1) - off;
    const unsigned bytes = (unsigned)min(sz, pkcap) * 4u;
    bulk_load(pkb + (size_t)buf * pkcap, S.pk + off, bytes, &mbar[warp][buf]);
  };
  int cur = 0;
  unsigned parity[3] = {0u, 0u, 0u};
  int first = -1;
  for (int l = 0; l < S.n_levels && first < 0; l++) {
    const int c = __ldg(S.lev_ptr + l) + warp;
    if (c < __ldg(S.lev_ptr + l + 1)) first = c;
  }
  if (first >= 0 && lane == 0) issue(first, 0);

  for (int lv = 0; lv < S.n_levels; lv++) {
    const int q0 = __ldg(S.lev_ptr + lv), q1 = __ldg(S.lev_ptr + lv + 1);
    for (int q = q0 + warp; q < q1; q += nw) {
      bool ok = mbar_wait(&mbar[warp][cur], parity[cur]);
      parity[cur] ^= 1u;
      const int nq = next_task(S, lv, q, warp, nw);
      if (nq >= 0 && lane == 0) issue(nq, cur ^ 1);
      if (!ok) atomicExch(&timed_out, 1);
      if (!ok || timed_out) { cur ^= 1; continue; }
      const int32_t* pk = pkb + (size_t)cur * pkcap;
      const int psz = __ldg(S.pk_off + q + 1) - __ldg(S.pk_off + q);
      const int k = pk[0], base = pk[1], ulen = pk[2], llen = pk[3];
      const int nA = pk[4], nops = pk[5], nbt = pk[6], nfw = pk[7], ob = pk[9];
      const int len = ulen + 1 + llen;
      const int32_t* fwp = pk + 12 + nA;
      const int32_t* btw = fwp + 2 * nfw;
      const int ops_at = 12 + nA + 2 * nfw + ((nbt + 3) >> 2);
      const bool ops_in_pk = (ops_at + 2 * nops) <= min(psz, pkcap);
      const bool in_smem = len <= cap;
      T* st = in_smem ? stage_w : (LUg + (size_t)base * 32u);
      T* stl = st + lane;
      // --- stage: one bulk copy of the column (A values / zeros)
      if (in_smem && lane == 0)
        bulk_load(stage_w, LUg + (size_t)base * 32u, (unsigned)len * 32u * sizeof(T), &mbar[warp][2]);
      // --- forward terms and b_k, first window of update values (cp.async)
      const bool in_dat = S.fuse_fwd && (2 * nfw + 1) <= dcap;
      if (in_dat) {
        for (int t = 0; t < nfw; t++) {
          cp_async_t<T>(dat + t * 32 + lane, LUg + (size_t)fwp[2 * t] * 32u + lane);
          cp_async_t<T>(dat + (nfw + t) * 32 + lane, X + xG + (size_t)fwp[2 * t + 1] * 32u + lane);
        }
        cp_async_t<T>(dat + 2 * nfw * 32 + lane, RHS + xG + (size_t)k * 32u + lane);
      }
      int ochunk = min(nops, opcap);
      const int32_t* dsrc = ops_in_pk ? pk + ops_at : opd;  // descriptors of the window
      if (!ops_in_pk) {
        // descriptors of the first window: lane-parallel coalesced loads
        for (int t = lane; t < ochunk; t += 32) {
          const uint32_t ps = __ldg(S.op_pos + ob + t);
          opd[2 * t] = __ldg(S.op_slot + ob + t) * 32;
          opd[2 * t + 1] = (int32_t)(((ps & 0xffffu) * 32u) | (((ps >> 16) * 32u) << 16));
        }
        __syncwarp();
      }
      for (int t = 0; t < ochunk; t++) cp_async_t<T>(opv + t * 32 + lane, LUg + dsrc[2 * t] + lane);
      asm volatile("cp.async.commit_group;\n" ::: "memory");
      if (in_smem) {
        if (!mbar_wait(&mbar[warp][2], parity[2])) atomicExch(&timed_out, 1);
        parity[2] ^= 1u;
      }
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      __syncwarp();
      // --- update batches
      int o = 0, cbase = 0;
      for (int b = 0; b < nbt; b++) {
        const int cnt = (btw[b >> 2] >> (8 * (b & 3))) & 0xff;
        if (o + cnt > cbase + ochunk) {  // refill the update window (long columns)
          cbase = o;
          ochunk = min(nops - o, opcap);
          __syncwarp();
          if (!ops_in_pk) {
            for (int t = lane; t < ochunk; t += 32) {
              const uint32_t ps = __ldg(S.op_pos + ob + o + t);
              opd[2 * t] = __ldg(S.op_slot + ob + o + t) * 32;
              opd[2 * t + 1] = (int32_t)(((ps & 0xffffu) * 32u) | (((ps >> 16) * 32u) << 16));
            }
            __syncwarp();
          }
          const int32_t* ds = ops_in_pk ? pk + ops_at + 2 * o : opd;
          for (int t = 0; t < ochunk; t++) cp_async_t<T>(opv + t * 32 + lane, LUg + ds[2 * t] + lane);
          cp_async_commit_wait();
          __syncwarp();
        }
        const int32_t* desc = ops_in_pk ? pk + ops_at + 2 * o : opd + 2 * (o - cbase);
        const T* ov = opv + (o - cbase) * 32 + lane;
        switch (cnt) {
          case 1: run_batch<T, 1>(stl, ov, desc); break;
          case 2: run_batch<T, 2>(stl, ov, desc); break;
          case 3: run_batch<T, 3>(stl, ov, desc); break;
          case 4: run_batch<T, 4>(stl, ov, desc); break;
          case 5: run_batch<T, 5>(stl, ov, desc); break;
          case 6: run_batch<T, 6>(stl, ov, desc); break;
          case 7: run_batch<T, 7>(stl, ov, desc); break;
          default: run_batch<T, 8>(stl, ov, desc); break;
        }
        o += cnt;
      }
      // --- pivot (static order), scale L, write back
      const T piv = stl[ulen * 32];
      if (piv == (T)0) bad = true;
      if (ptol > 0.0f) {
        T colmax = fabs(piv);
        for (int t = 0; t < llen; t++) colmax = fmax(colmax, fabs(stl[(ulen + 1 + t) * 32]));
        if ((float)fabs(piv) < ptol * (float)colmax) tiny = true;
      }
      const T inv = (T)1 / piv;
      T* dstl = LUg + (size_t)base * 32u + lane;
      if (in_smem)
        for (int p = 0; p <= ulen; p++) dstl[p * 32] = stl[p * 32];
      for (int p = ulen + 1; p < len; p++) dstl[p * 32] = stl[p * 32] * inv;
      if (S.fuse_fwd) {
        T y;
        if (in_dat) {
          y = dat[2 * nfw * 32 + lane];
          for (int t = 0; t < nfw; t++) y -= dat[t * 32 + lane] * dat[(nfw + t) * 32 + lane];
        } else {
          y = RHS[xG + (size_t)k * 32u + lane];
          for (int t0 = 0; t0 < nfw; t0 += 16) {
            T c[16], xv[16];
#pragma unroll
            for (int t = 0; t < 16; t++)
              if (t0 + t < nfw) {
                c[t] = LUg[(size_t)fwp[2 * (t0 + t)] * 32u + lane];
                xv[t] = X[xG + (size_t)fwp[2 * (t0 + t) + 1] * 32u + lane];
              }
#pragma unroll
            for (int t = 0; t < 16; t++)
              if (t0 + t < nfw) y -= c[t] * xv[t];
          }
        }
        X[xG + (size_t)k * 32u + lane] = y;
      }
      __syncwarp();
      cur ^= 1;
    }
    __syncthreads();
  }
  if (bad) atomicOr(&flags[0][lane], 1);
  if (tiny) atomicOr(&flags[1][lane], 1);
  __syncthreads();
  if (warp == 0) {
    if (flags[0][lane]) D.sing[s] = 1;
    if (flags[1][lane]) D.piv_flag[s] = 1;
    if (lane == 0 && timed_out && D.err) atomicExch(D.err, 1);
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
