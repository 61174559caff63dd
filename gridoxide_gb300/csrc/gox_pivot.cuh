// FP64 threshold-partial-pivoting factorization and solve on the GPU, for
// the scenarios of a mixed-precision batch whose FP32 refactor met a pivot
// below the pivot-ratio threshold.  Their static pivot order is poor for
// their own Jacobian, so each of their Newton steps factors that Jacobian
// afresh, choosing pivots as KLU does: Gilbert-Peierls left-looking LU per
// BTF block (src/klu_native/kernel.rs:341-416 factor_block: depth-first
// reach of each column in the graph of the finished L columns, sparse
// triangular solve in topological order, then lpivot, kernel.rs:187-262:
// the diagonal row when |x_diag| >= tol * max |x|, else the largest, with
// KLU's bookkeeping of which row counts as each column's diagonal), and
// the block back substitution with the off-diagonal part
// (src/klu_native/solve.rs:56-102).  Pruning of L columns is omitted: it
// only shortens the depth-first searches.
//
// One warp per scenario: lane 0 runs the searches and the pivot choice,
// the 32 lanes the column updates, scalings and copies.  The scenario's
// factor lives in its own scratch (patterns with a reserved fill bound);
// a factor that would exceed the bound, a zero pivot or a non-finite
// solution marks the scenario singular.  The Jacobian values are read from
// the batch's fill image (the static layout's LU slots and off-diagonal
// entries), the right-hand side from the static rhs layout, and the
// solution is written where the static path writes it, so the rest of the
// Newton loop is unchanged.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "gox_kernels.cuh"

namespace gox {

struct PivotDev {
  int n, nblocks, n_slots, n_off;
  int lcap, ucap, ocap;
  const int32_t* R;        // [nblocks + 1] block bounds (factor column order)
  const int32_t* cp;       // [n + 1] A entries of factor column k ...
  const int32_t* ci;       // ... their row in the BTF-permuted row order
  const int32_t* csrc;     // ... where the fill writes their value: >= 0 an LU
                           //     slot of the static layout, < 0 -(off entry + 1)
  const int32_t* rhs_pos;  // [n] static right-hand-side position of permuted row i
  double tol;              // pivot tolerance (KLU's default 0.001)
  unsigned char* scratch;  // per CTA: its scenario's factor and work arrays
  size_t stride;           // bytes per CTA
};

// Scratch of one scenario, carved in this order (16-byte aligned pieces).
struct PivotWork {
  double *X, *bp, *Ud, *Lx, *Ux, *Ox;
  int32_t *pinv, *pb, *flag, *stack, *dstk, *dpos, *lrows, *Lp, *Up, *Op, *Li, *Ui, *Oi;
};

__host__ __device__ inline size_t pivot_piece(size_t bytes) { return (bytes + 15) & ~(size_t)15; }

__host__ __device__ inline size_t pivot_stride(int n, int lcap, int ucap, int ocap) {
  const size_t d = 8, i = 4;
  return pivot_piece(d * n) * 3 + pivot_piece(d * lcap) + pivot_piece(d * ucap) +
         pivot_piece(d * ocap) + pivot_piece(i * n) * 7 + pivot_piece(i * (n + 1)) * 3 +
         pivot_piece(i * lcap) + pivot_piece(i * ucap) + pivot_piece(i * ocap);
}

__device__ inline PivotWork pivot_work(const PivotDev& P, unsigned char* b) {
  PivotWork W;
  size_t o = 0;
  auto dp = [&](size_t cnt) {
    double* p = reinterpret_cast<double*>(b + o);
    o += pivot_piece(8 * cnt);
    return p;
  };
  auto ip = [&](size_t cnt) {
    int32_t* p = reinterpret_cast<int32_t*>(b + o);
    o += pivot_piece(4 * cnt);
    return p;
  };
  const int n = P.n;
  W.X = dp(n); W.bp = dp(n); W.Ud = dp(n);
  W.Lx = dp(P.lcap); W.Ux = dp(P.ucap); W.Ox = dp(P.ocap);
  W.pinv = ip(n); W.pb = ip(n); W.flag = ip(n); W.stack = ip(n); W.dstk = ip(n); W.dpos = ip(n);
  W.lrows = ip(n);
  W.Lp = ip(n + 1); W.Up = ip(n + 1); W.Op = ip(n + 1);
  W.Li = ip(P.lcap); W.Ui = ip(P.ucap); W.Oi = ip(P.ocap);
  return W;
}

__device__ __forceinline__ int pv_flip(int i) { return -i - 2; }

// grid: CTAs of one warp, each looping over scenarios s = blockIdx.x,
// blockIdx.x + gridDim.x, ... of the batch (the running ones only).
__global__ void __launch_bounds__(32) k_factor_pivot(PivotDev P, BatchDev D) {
  const int lane = threadIdx.x;
  PivotWork W = pivot_work(P, P.scratch + (size_t)blockIdx.x * P.stride);
  const int n = P.n;
  const double* img = (const double*)D.lu;
  const double* offimg = (const double*)D.off;
  const double* rhs = (const double*)D.rhs;
  double* sol = (double*)D.sol;
  __shared__ int sh_top, sh_nl, sh_bad, sh_ppiv;
  for (int s = blockIdx.x; s < D.G * 32; s += gridDim.x) {
    const int g = s >> 5, l = s & 31;
    if (!D.gact[g] || D.status[s] != ST_RUNNING || D.sing[s] != 0) continue;
    auto aval = [&](int src) -> double {
      return src >= 0 ? img[((size_t)g * P.n_slots + src) * 32u + l]
                      : offimg[((size_t)g * P.n_off + (size_t)(-src - 1)) * 32u + l];
    };
    for (int i = lane; i < n; i += 32) {
      W.X[i] = 0.0;
      W.flag[i] = -1;
    }
    if (lane == 0) {
      W.Lp[0] = 0;
      W.Up[0] = 0;
      W.Op[0] = 0;
      sh_bad = 0;
    }
    __syncwarp();
    for (int b = 0; b < P.nblocks; b++) {
      const int k1 = P.R[b], k2 = P.R[b + 1];
      for (int i = k1 + lane; i < k2; i += 32) {
        W.pinv[i] = pv_flip(i);  // row i is the diagonal of column i
        W.pb[i] = i;
      }
      __syncwarp();
      for (int k = k1; k < k2; k++) {
        if (lane == 0) {
          // reach of column k: rows of A(:, k) in this block, and through
          // the finished columns' L patterns (depth first, iterative);
          // pivotal rows go to the stack's top part in topological order,
          // the others to lrows
          int top = n, nl = 0, no = W.Op[k];
          for (int p = P.cp[k]; p < P.cp[k + 1]; p++) {
            const int i0 = P.ci[p];
            if (i0 < k1) {  // an entry of an earlier block: off-diagonal part
              if (no < P.ocap) {
                W.Oi[no] = i0;
                W.Ox[no] = aval(P.csrc[p]);
              }
              no++;
              continue;
            }
            if (W.flag[i0] == k) continue;
            W.flag[i0] = k;
            if (W.pinv[i0] < 0) {
              W.lrows[nl++] = i0;
              continue;
            }
            int head = 0;
            W.dstk[0] = i0;
            W.dpos[0] = W.Lp[W.pinv[i0]];
            while (head >= 0) {
              const int j = W.dstk[head];
              const int pe = W.Lp[W.pinv[j] + 1];
              int q = W.dpos[head];
              bool down = false;
              for (; q < pe; q++) {
                const int r = W.Li[q];
                if (W.flag[r] == k) continue;
                W.flag[r] = k;
                if (W.pinv[r] >= 0) {
                  W.dpos[head] = q + 1;
                  W.dstk[++head] = r;
                  W.dpos[head] = W.Lp[W.pinv[r]];
                  down = true;
                  break;
                }
                W.lrows[nl++] = r;
              }
              if (!down) {
                head--;
                W.stack[--top] = j;
              }
            }
          }
          if (no > P.ocap) sh_bad = 1;
          W.Op[k + 1] = no < P.ocap ? no : P.ocap;
          sh_top = top;
          sh_nl = nl;
        }
        __syncwarp();
        const int top = sh_top, nl = sh_nl;
        if (sh_bad) break;
        // the column's values (A entries of this block)
        for (int p = P.cp[k] + lane; p < P.cp[k + 1]; p += 32) {
          const int i0 = P.ci[p];
          if (i0 >= k1) W.X[i0] = aval(P.csrc[p]);
        }
        __syncwarp();
        // sparse triangular solve with the finished columns, in topological order
        for (int q = top; q < n; q++) {
          const int j = W.stack[q];
          const int jc = W.pinv[j];
          const double xj = W.X[j];
          for (int p = W.Lp[jc] + lane; p < W.Lp[jc + 1]; p += 32) W.X[W.Li[p]] -= W.Lx[p] * xj;
          __syncwarp();
        }
        if (lane == 0) {
          // lpivot: the largest candidate (first in discovery order on ties),
          // unless the diagonal row is within the tolerance of it
          const int diagrow = W.pb[k];
          double amax = -1.0;
          int ppiv = -1, pdiag = -1;
          for (int t = 0; t < nl; t++) {
            const int i = W.lrows[t];
            const double a = fabs(W.X[i]);
            if (i == diagrow) pdiag = t;
            if (a > amax) {
              amax = a;
              ppiv = t;
            }
          }
          if (pdiag >= 0 && fabs(W.X[diagrow]) >= P.tol * amax) ppiv = pdiag;
          const bool room = W.Lp[k] + nl - 1 <= P.lcap && W.Up[k] + (n - top) <= P.ucap;
          if (ppiv < 0 || W.X[W.lrows[ppiv]] == 0.0 || !room) sh_bad = 1;
          sh_ppiv = ppiv;
        }
        __syncwarp();
        if (sh_bad) break;
        const int ppiv = sh_ppiv;
        const int pivrow = W.lrows[ppiv];
        const double pivot = W.X[pivrow];
        __syncwarp();
        // L(:, k) = the other candidates / pivot; U(:, k) = the reach
        for (int t = lane; t < nl; t += 32) {
          if (t == ppiv) continue;
          const int i = W.lrows[t];
          const int dst = W.Lp[k] + (t < ppiv ? t : t - 1);
          W.Li[dst] = i;
          W.Lx[dst] = W.X[i] / pivot;
        }
        for (int q = top + lane; q < n; q += 32) {
          const int j = W.stack[q];
          W.Ui[W.Up[k] + (q - top)] = W.pinv[j];
          W.Ux[W.Up[k] + (q - top)] = W.X[j];
        }
        __syncwarp();
        for (int t = lane; t < nl; t += 32) W.X[W.lrows[t]] = 0.0;
        for (int q = top + lane; q < n; q += 32) W.X[W.stack[q]] = 0.0;
        __syncwarp();
        if (lane == 0) {
          W.Ud[k] = pivot;
          const int diagrow = W.pb[k];
          if (pivrow != diagrow && W.pinv[diagrow] < 0) {
            // the pivot row was the diagonal of a later column: that column
            // takes this column's diagonal row instead
            const int kbar = pv_flip(W.pinv[pivrow]);
            W.pb[kbar] = diagrow;
            W.pinv[diagrow] = pv_flip(kbar);
          }
          W.pb[k] = pivrow;
          W.pinv[pivrow] = k;
          W.Lp[k + 1] = W.Lp[k] + nl - 1;
          W.Up[k + 1] = W.Up[k] + (n - top);
        }
        __syncwarp();
      }
      if (sh_bad) break;
    }
    if (sh_bad) {
      if (lane == 0) D.sing[s] = 1;
      __syncwarp();
      continue;
    }
    // solve: b in pivot order, then the blocks in reverse: unit-L forward,
    // U backward (column oriented), then the off-diagonal part of the
    // block's columns moves to the earlier blocks' right-hand sides
    for (int k = lane; k < n; k += 32)
      W.bp[k] = rhs[((size_t)g * n + (size_t)P.rhs_pos[W.pb[k]]) * 32u + l];
    __syncwarp();
    for (int b = P.nblocks - 1; b >= 0; b--) {
      const int k1 = P.R[b], k2 = P.R[b + 1];
      for (int k = k1; k < k2; k++) {
        const double xk = W.bp[k];
        for (int p = W.Lp[k] + lane; p < W.Lp[k + 1]; p += 32) W.bp[W.pinv[W.Li[p]]] -= W.Lx[p] * xk;
        __syncwarp();
      }
      for (int k = k2 - 1; k >= k1; k--) {
        const double xk = W.bp[k] / W.Ud[k];
        __syncwarp();
        if (lane == 0) W.bp[k] = xk;
        for (int p = W.Up[k] + lane; p < W.Up[k + 1]; p += 32) W.bp[W.Ui[p]] -= W.Ux[p] * xk;
        __syncwarp();
      }
      for (int k = k1; k < k2; k++) {
        const double xk = W.bp[k];
        for (int p = W.Op[k] + lane; p < W.Op[k + 1]; p += 32) W.bp[W.pinv[W.Oi[p]]] -= W.Ox[p] * xk;
        __syncwarp();
      }
    }
    bool bad = false;
    for (int k = lane; k < n; k += 32) {
      const double x = W.bp[k];
      bad |= !isfinite(x);
      sol[((size_t)g * n + k) * 32u + l] = x;
    }
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0 && bad) D.sing[s] = 1;
    __syncwarp();
  }
}

}  // namespace gox
