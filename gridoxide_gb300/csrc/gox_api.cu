// extern "C" layer and device engine of the GB300 batched power-flow
// library.  See include/gridoxide_gb300.h for the contract of each entry
// point and the reference interface it replaces.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <type_traits>
#include <atomic>
#include <cmath>
#include <functional>
#include <map>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gridoxide_gb300.h"
#include "gox_engine.hpp"
#include "gox_stream.hpp"
#include "gox_kernels.cuh"
#include "gox_pivot.cuh"

namespace gox {

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define GOX_CK(x)                                                                          \
  do {                                                                                     \
    cudaError_t e_ = (x);                                                                  \
    if (e_ != cudaSuccess)                                                                 \
      throw CudaError(std::string(#x) + ": " + cudaGetErrorString(e_));                    \
  } while (0)

// The stream of the entry point running on this thread: device buffers are
// allocated and freed in its order (cudaMallocAsync / cudaFreeAsync) while it
// is set.  A plain cudaFree synchronizes the whole device, which would stall
// every other solve in flight (concurrent topologies, the server's workers).
static thread_local cudaStream_t tl_alloc_stream = nullptr;
struct AllocStreamScope {
  cudaStream_t prev;
  explicit AllocStreamScope(cudaStream_t s) : prev(tl_alloc_stream) { tl_alloc_stream = s; }
  ~AllocStreamScope() { tl_alloc_stream = prev; }
};

// Owning device allocation.
struct DevMem {
  void* p = nullptr;
  size_t bytes = 0;
  bool pooled = false;  // from cudaMallocAsync: may be freed in stream order
  DevMem() = default;
  DevMem(const DevMem&) = delete;
  DevMem& operator=(const DevMem&) = delete;
  ~DevMem() { release(); }
  void release() {
    if (p) {
      if (pooled && tl_alloc_stream) cudaFreeAsync(p, tl_alloc_stream);
      else cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
    pooled = false;
  }
  void ensure(size_t b) {
    if (b <= bytes && p) return;
    // a buffer that has to grow grows by half again at least: fewer
    // reallocations as batches vary
    if (p) b = std::max(b, bytes + bytes / 2);
    release();
    if (b == 0) b = 16;
    pooled = tl_alloc_stream != nullptr;
    cudaError_t e = pooled ? cudaMallocAsync(&p, b, tl_alloc_stream) : cudaMalloc(&p, b);
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      throw std::bad_alloc();
    }
    GOX_CK(e);
    bytes = b;
  }
  template <typename T>
  T* as() const { return reinterpret_cast<T*>(p); }
};

template <typename T>
static void upload(DevMem& m, const std::vector<T>& v) {
  m.ensure(sizeof(T) * std::max<size_t>(v.size(), 1));
  if (v.empty()) return;
  if (m.pooled) {  // usable in the order of the stream it was allocated on
    GOX_CK(cudaMemcpyAsync(m.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice,
                           tl_alloc_stream));
    GOX_CK(cudaStreamSynchronize(tl_alloc_stream));
  } else {
    GOX_CK(cudaMemcpy(m.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  }
}

// ---------------------------------------------------------------------------
// Layout kernels: row-major [B][N] <-> scenario-interleaved [G][N][32].

__global__ void k_scatter_rows(const double* __restrict__ src, int B, int N, int stride,
                               double* __restrict__ dst, int G) {
  // dst[(g*N + i)*32 + l] = src[s*stride + i], s = min(32g + l, B-1)
  size_t total = (size_t)G * N * 32;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    int l = (int)(t & 31);
    size_t gi = t >> 5;
    int i = (int)(gi % N);
    int g = (int)(gi / N);
    int s = min(g * 32 + l, B - 1);
    dst[t] = src[(size_t)s * stride + i];
  }
}

__global__ void k_gather_rows(const double* __restrict__ src, int B, int N, int G,
                              double* __restrict__ dst) {
  size_t total = (size_t)B * N;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    int s = (int)(t / N);
    int i = (int)(t % N);
    int g = s >> 5, l = s & 31;
    dst[t] = src[((size_t)g * N + i) * 32 + l];
  }
}

// Re-packing: the running scenarios of a batch (from[k], k < R) moved into
// the first lanes of a smaller batch of Gp groups, and back.  Slots from R
// up to whole groups copy scenario from[R - 1] and are marked unused.
// Interleaved arrays [G][rows][32] of 4- or 8-byte words:
template <typename W>
__global__ void k_pack_rows(const W* __restrict__ src, W* __restrict__ dst, int rows,
                            const int32_t* __restrict__ from, int R, int Gp) {
  const size_t total = (size_t)Gp * rows * 32;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t gr = t >> 5;  // packed group * rows + row
    const int k = (int)(gr / rows) * 32 + (int)(t & 31);
    const int r = (int)(gr % rows);
    const int s = from[min(k, R - 1)];
    dst[t] = src[((size_t)(s >> 5) * rows + r) * 32 + (s & 31)];
  }
}
template <typename W>
__global__ void k_unpack_rows(const W* __restrict__ src, W* __restrict__ dst, int rows,
                              const int32_t* __restrict__ from, int R) {
  const size_t total = (size_t)R * rows;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / R), k = (int)(t % R), s = from[k];
    dst[((size_t)(s >> 5) * rows + r) * 32 + (s & 31)] =
        src[((size_t)(k >> 5) * rows + r) * 32 + (k & 31)];
  }
}
// Per-scenario arrays of `width` words (scenario s at s * width):
template <typename W>
__global__ void k_pack_flat(const W* __restrict__ src, W* __restrict__ dst, int width,
                            const int32_t* __restrict__ from, int R, int K) {
  const size_t total = (size_t)K * width;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / width), c = (int)(t % width);
    dst[t] = src[(size_t)from[min(k, R - 1)] * width + c];
  }
}
template <typename W>
__global__ void k_unpack_flat(const W* __restrict__ src, W* __restrict__ dst, int width,
                              const int32_t* __restrict__ from, int R) {
  const size_t total = (size_t)R * width;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / width), c = (int)(t % width);
    dst[(size_t)from[k] * width + c] = src[t];
  }
}
// The packed batch's padding slots do not run; every packed group runs.
__global__ void k_pack_mark(int32_t* __restrict__ status, int32_t* __restrict__ gact, int R,
                            int Gp) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < Gp * 32 && t >= R) status[t] = ST_UNUSED;
  if (t < Gp) gact[t] = 1;
}

// Uniformly scaled injections: p[s][i] = p_base[i] * scale[s] (and q), the
// scenarios of uniform_load_scaling (src/batch.rs:98-106; a bus with no
// injection stays at zero either way)
__global__ void k_scale_rows(const double* __restrict__ p_base, const double* __restrict__ q_base,
                             const double* __restrict__ scale, int B, int N, double* __restrict__ p,
                             double* __restrict__ q) {
  const size_t total = (size_t)B * N;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(t / N), i = (int)(t % N);
    const double f = scale[s];
    p[t] = p_base[i] * f;
    q[t] = q_base[i] * f;
  }
}

// dst row r = src row idx[r] (rows of `w` elements of 4 or 8 bytes), and back
template <typename E>
__global__ void k_take_rows(const E* __restrict__ src, int w, const int32_t* __restrict__ idx,
                            int nr, E* __restrict__ dst) {
  const size_t total = (size_t)nr * w;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = t / w, c = t % w;
    dst[t] = src[(size_t)idx[r] * w + c];
  }
}
template <typename E>
__global__ void k_put_rows(const E* __restrict__ src, int w, const int32_t* __restrict__ idx,
                           int nr, E* __restrict__ dst) {
  const size_t total = (size_t)nr * w;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t r = t / w, c = t % w;
    dst[(size_t)idx[r] * w + c] = src[t];
  }
}

__global__ void k_init_scen(int B, int G, int32_t* status, int32_t* iters, int32_t* sing,
                            int32_t* piv, double* maxmis, unsigned long long* maxacc) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= G * 32) return;
  status[s] = (s < B) ? ST_RUNNING : ST_UNUSED;
  iters[s] = 0;
  sing[s] = 0;
  piv[s] = 0;
  maxmis[s] = 0.0;
  maxacc[s] = 0ull;
}

// Outage slots -> branch buses; validates the slots.  err[0] set on a bad slot.
__global__ void k_outage_prep(int B, int G, const int32_t* slot_in, const double* dre_in,
                              const double* dim_in, const int32_t* yp, const int32_t* yi, int n,
                              int nnz, int32_t* o_slot, double* o_dre, double* o_dim,
                              int32_t* o_bf, int32_t* o_bt, int32_t* err) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= G * 32) return;
  int src = min(s, B - 1);
  bool use = (s < B) && slot_in[4 * src] >= 0;
  int sl[4];
  for (int c = 0; c < 4; c++) sl[c] = use ? slot_in[4 * src + c] : -1;
  int bf = -1, bt = -1;
  if (use) {
    for (int c = 0; c < 4; c++)
      if (sl[c] < 0 || sl[c] >= nnz) { atomicExch(err, 1); use = false; }
  }
  if (use) {
    // row of a slot: binary search in the row pointers
    auto row_of = [&](int sp) {
      int lo = 0, hi = n - 1;
      while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (yp[mid] <= sp) lo = mid; else hi = mid - 1;
      }
      return lo;
    };
    bf = row_of(sl[0]);
    bt = row_of(sl[3]);
    // (ff, ft, tf, tt) must be (f,f), (f,t), (t,f), (t,t)
    if (yi[sl[0]] != bf || yi[sl[3]] != bt || row_of(sl[1]) != bf || yi[sl[1]] != bt ||
        row_of(sl[2]) != bt || yi[sl[2]] != bf) {
      atomicExch(err, 1);
      use = false;
      bf = bt = -1;
    }
  }
  o_bf[s] = use ? bf : -1;
  o_bt[s] = use ? bt : -1;
  for (int c = 0; c < 4; c++) {
    o_slot[4 * s + c] = use ? sl[c] : -1;
    o_dre[4 * s + c] = use ? dre_in[4 * src + c] : 0.0;
    o_dim[4 * s + c] = use ? dim_in[4 * src + c] : 0.0;
  }
}

__global__ void k_unpack_scen(int B, const int32_t* st_in, const int32_t* it_in,
                              const double* mm_in, const double* hist_in, int max_iter,
                              int32_t* st, int32_t* it, double* mm, double* hist) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  st[s] = st_in[s];
  it[s] = it_in[s];
  mm[s] = mm_in[s];
  if (hist)
    for (int k = 0; k < max_iter; k++) hist[(size_t)s * max_iter + k] = hist_in[(size_t)s * max_iter + k];
}

// ---------------------------------------------------------------------------

struct DevSchedule {
  DevMem yp, yi, yre, yim, bus_rowP, bus_rowQ, bus_colA, bus_colV, a_kind, a_bi, a_bk, a_yslot,
      a_dst, lev_ptr, lev_cols, c_base, c_ulen, c_llen, c_abeg, c_aend, op_ptr, op_slot, op_pos, ph_ptr,
      ph_rows, ph_kind, fw_ptr, fw_slot, fw_col, bw_ptr, bw_slot, bw_col, diag_slot, bt_ptr, bt_cnt,
      pk_off, pk, slot_a, off_a, ft_dst, ft_bus, ft_y, ft_yf, fz_slot;
  SchedDev d{};
  int max_collen = 0, max_ops = 0, max_pk = 0, max_head = 0, max_fw = 0;
  // refactor command streams, FP32 and FP64 plans
  DevMem sw[2], sc0[2], snc[2];
  StreamDev st[2]{};
  int st_nw[2] = {0, 0};
  size_t st_smem[2] = {0, 0};
  bool st_bwd[2] = {false, false};  // the stream runs the backward substitution too
  int st_wl[2] = {0, 0}, st_wp[2] = {0, 0};  // levels / phases the wide kernels run
  int st_wr[2] = {0, 0};                      // their stage rows per warp
  std::vector<int32_t> lev_ptr_h;  // host copy: columns per refactor level
  // launches of one refactor (with both substitutions when the stream has them)
  int refactor_launches(int i) const { return 1 + st_wl[i] + st_wp[i]; }

  void load_streams(const Stream& s32, const Stream& s64) {
    const Stream* ss[2] = {&s32, &s64};
    for (int i = 0; i < 2; i++) {
      upload(sw[i], ss[i]->words);
      upload(sc0[i], ss[i]->chunk0);
      upload(snc[i], ss[i]->nchunks);
      st[i].words = sw[i].as<int32_t>();
      st[i].chunk0 = sc0[i].as<int32_t>();
      st[i].nchunks = snc[i].as<int32_t>();
      st[i].ring_rows = ss[i]->plan.ring_rows;
      st[i].rows_total = ring_total(ss[i]->plan);
      st[i].chunk_words = ss[i]->plan.chunk_words;
      st[i].n_bars = ss[i]->n_bars;
      st[i].sync = ss[i]->plan.sync;
      st_nw[i] = ss[i]->plan.nw;
      st_smem[i] = stream_smem_bytes(ss[i]->plan);
      st_bwd[i] = ss[i]->has_bwd;
      st_wl[i] = ss[i]->plan.wide_levels;
      st_wp[i] = ss[i]->plan.wide_phases;
      st_wr[i] = ss[i]->plan.wide_rows;
    }
  }

  void load(const Schedule& sc, const std::vector<int32_t>& yp_h, const std::vector<int32_t>& yi_h,
            const std::vector<double>& yre_h, const std::vector<double>& yim_h) {
    upload(yp, yp_h); upload(yi, yi_h); upload(yre, yre_h); upload(yim, yim_h);
    upload(bus_rowP, sc.bus_rowP); upload(bus_rowQ, sc.bus_rowQ);
    upload(bus_colA, sc.bus_colA); upload(bus_colV, sc.bus_colV);
    upload(a_kind, sc.a_kind); upload(a_bi, sc.a_bi); upload(a_bk, sc.a_bk);
    upload(a_yslot, sc.a_yslot); upload(a_dst, sc.a_dst);
    upload(lev_ptr, sc.lev_ptr); upload(lev_cols, sc.lev_cols); upload(c_base, sc.c_base);
    lev_ptr_h = sc.lev_ptr;
    upload(c_ulen, sc.c_ulen); upload(c_llen, sc.c_llen); upload(c_abeg, sc.c_abeg);
    upload(c_aend, sc.c_aend);
    upload(op_ptr, sc.op_ptr); upload(op_slot, sc.op_slot); upload(op_pos, sc.op_pos);
    upload(ph_ptr, sc.ph_ptr); upload(ph_rows, sc.ph_rows); upload(ph_kind, sc.ph_kind);
    upload(fw_ptr, sc.fw_ptr); upload(fw_slot, sc.fw_slot); upload(fw_col, sc.fw_col);
    upload(bw_ptr, sc.bw_ptr); upload(bw_slot, sc.bw_slot); upload(bw_col, sc.bw_col);
    upload(diag_slot, sc.diag_slot);
    upload(bt_ptr, sc.bt_ptr); upload(bt_cnt, sc.bt_cnt);
    upload(pk_off, sc.pk_off); upload(pk, sc.pk);
    upload(slot_a, sc.slot_a); upload(off_a, sc.off_a);
    {
      // fill tasks: one per Y entry (i, k) with Jacobian entries, holding the
      // destinations of its H, N, M, L entries (diagonal tasks first), then
      // the zero fill-in slots of the factor (power-flow topologies only: a
      // linear-solver handle has no Y and no Jacobian kinds)
      const bool pf = !yre_h.empty();
      std::vector<int32_t> dst_of_a(sc.n_a, -1);
      std::vector<int32_t> zeros;
      for (int x = 0; pf && x < sc.n_slots; x++) {
        if (sc.slot_a[x] >= 0) dst_of_a[sc.slot_a[x]] = x;
        else zeros.push_back(x);
      }
      for (int j = 0; pf && j < sc.n_off; j++) dst_of_a[sc.off_a[j]] = sc.n_slots + j;
      std::map<std::pair<int, int>, int> task_of;
      std::vector<int32_t> tdst, tbus;
      std::vector<double> ty;
      std::vector<float> tyf;
      auto quad = [](int kind) { return kind == 0 || kind == 2 ? 0 : kind == 1 || kind == 3 ? 1
                                        : kind == 4 || kind == 6 ? 2 : 3; };
      for (int pass = 0; pf && pass < 2; pass++) {  // diagonal tasks, then off-diagonal ones
        for (int a = 0; a < sc.n_a; a++) {
          const int kind = sc.a_kind[a];
          const bool diag = kind == 0 || kind == 1 || kind == 4 || kind == 5;
          if (diag != (pass == 0)) continue;
          const int bi = sc.a_bi[a], bk = diag ? sc.a_bi[a] : sc.a_bk[a];
          auto it = task_of.find({bi, bk});
          int t;
          if (it == task_of.end()) {
            t = (int)(tbus.size() / 4);
            task_of[{bi, bk}] = t;
            tdst.insert(tdst.end(), {-1, -1, -1, -1});
            tbus.insert(tbus.end(), {bi, bk, sc.a_yslot[a], diag ? 1 : 0});
            const double yr = yre_h[sc.a_yslot[a]], yi = yim_h[sc.a_yslot[a]];
            ty.insert(ty.end(), {yr, yi});
            tyf.insert(tyf.end(), {(float)yr, (float)yi});
          } else {
            t = it->second;
            if (tbus[(size_t)t * 4 + 2] != sc.a_yslot[a])
              throw std::logic_error("Jacobian entries of one bus pair on two Y slots");
          }
          int32_t& d = tdst[(size_t)t * 4 + quad(kind)];
          if (d != -1) throw std::logic_error("two Jacobian entries of one kind and bus pair");
          d = dst_of_a[a];
        }
      }
      upload(ft_dst, tdst);
      upload(ft_bus, tbus);
      upload(ft_y, ty);
      upload(ft_yf, tyf);
      upload(fz_slot, zeros);
      d.n_ftask = (int)(tbus.size() / 4);
      d.n_fzero = (int)zeros.size();
      d.ft_dst = reinterpret_cast<const int4*>(ft_dst.p);
      d.ft_bus = reinterpret_cast<const int4*>(ft_bus.p);
      d.ft_y = reinterpret_cast<const double2*>(ft_y.p);
      d.ft_yf = reinterpret_cast<const float2*>(ft_yf.p);
      d.fz_slot = fz_slot.as<int32_t>();
    }
    d.slot_a = slot_a.as<int32_t>(); d.off_a = off_a.as<int32_t>();
    d.n_off_real = sc.n_off;
    d.bt_ptr = bt_ptr.as<int32_t>(); d.bt_cnt = bt_cnt.as<uint8_t>();
    d.pk_off = pk_off.as<int32_t>(); d.pk = pk.as<int32_t>();
    max_collen = sc.max_collen; max_ops = sc.max_ops; max_pk = sc.max_pk;
    max_head = sc.max_head; max_fw = sc.max_fw;
    d.n_bus = sc.n_bus; d.n_u = sc.n_u; d.n_a = sc.n_a; d.n_slots = sc.n_slots;
    d.n_off = std::max(sc.n_off, 1); d.n_levels = sc.n_levels; d.n_phases = sc.n_phases;
    d.nnz_y = (int)yi_h.size();
    d.fuse_fwd = sc.fuse_fwd ? 1 : 0;
    d.yp = yp.as<int32_t>(); d.yi = yi.as<int32_t>(); d.yre = yre.as<double>(); d.yim = yim.as<double>();
    d.bus_rowP = bus_rowP.as<int32_t>(); d.bus_rowQ = bus_rowQ.as<int32_t>();
    d.bus_colA = bus_colA.as<int32_t>(); d.bus_colV = bus_colV.as<int32_t>();
    d.a_kind = a_kind.as<int32_t>(); d.a_bi = a_bi.as<int32_t>(); d.a_bk = a_bk.as<int32_t>();
    d.a_yslot = a_yslot.as<int32_t>(); d.a_dst = a_dst.as<int32_t>();
    d.lev_ptr = lev_ptr.as<int32_t>(); d.lev_cols = lev_cols.as<int32_t>();
    d.c_base = c_base.as<int32_t>(); d.c_ulen = c_ulen.as<int32_t>(); d.c_llen = c_llen.as<int32_t>();
    d.c_abeg = c_abeg.as<int32_t>(); d.c_aend = c_aend.as<int32_t>(); d.op_ptr = op_ptr.as<int32_t>();
    d.op_slot = op_slot.as<int32_t>(); d.op_pos = op_pos.as<uint32_t>();
    d.ph_ptr = ph_ptr.as<int32_t>(); d.ph_rows = ph_rows.as<int32_t>(); d.ph_kind = ph_kind.as<int32_t>();
    d.fw_ptr = fw_ptr.as<int32_t>(); d.fw_slot = fw_slot.as<int32_t>(); d.fw_col = fw_col.as<int32_t>();
    d.bw_ptr = bw_ptr.as<int32_t>(); d.bw_slot = bw_slot.as<int32_t>(); d.bw_col = bw_col.as<int32_t>();
    d.diag_slot = diag_slot.as<int32_t>();
  }
};

// Device buffers of one batch (capacity in groups of 32 scenarios).
struct DevBatch {
  int G = 0, prec = -1, max_iter = 0;
  DevMem vm, va, e, f, psp, qsp, cth, sth, eT, fT, ivT, pT, qT, jbuf, lu, off, rhs, sol;
  DevMem status, iters, sing, piv, maxmis, maxacc, hist, gact, nactive, err;
  DevMem o_slot, o_bf, o_bt, o_dre, o_dim;
  DevMem in_stage, out_stage;  // host I/O staging (row-major)

  std::vector<DevMem*> all() {
    return {&vm, &va, &e, &f, &psp, &qsp, &cth, &sth, &eT, &fT, &ivT, &pT, &qT, &jbuf, &lu, &off,
            &rhs, &sol, &status, &iters, &sing, &piv, &maxmis, &maxacc, &hist, &gact, &nactive,
            &err, &o_slot, &o_bf, &o_bt, &o_dre, &o_dim, &in_stage, &out_stage};
  }
  size_t bytes() {
    size_t b = 0;
    for (DevMem* m : all()) b += m->bytes;
    return b;
  }
  void release() {
    for (DevMem* m : all()) m->release();
    G = 0;
  }

  void ensure(const SchedDev& S, int G_, int prec_, int max_iter_, bool want_hist) {
    const size_t nb = (size_t)G_ * S.n_bus * 32, w = prec_ == GOX_PRECISION_FP64 ? 8 : 4;
    vm.ensure(nb * 8); va.ensure(nb * 8); e.ensure(nb * 8); f.ensure(nb * 8);
    psp.ensure(nb * 8); qsp.ensure(nb * 8); cth.ensure(nb * 8); sth.ensure(nb * 8);
    eT.ensure(nb * w); fT.ensure(nb * w); ivT.ensure(nb * w); pT.ensure(nb * w); qT.ensure(nb * w);
    jbuf.ensure((size_t)G_ * S.n_a * 32 * w);
    lu.ensure((size_t)G_ * S.n_slots * 32 * w);
    off.ensure((size_t)G_ * S.n_off * 32 * w);
    rhs.ensure((size_t)G_ * S.n_u * 32 * w);
    sol.ensure((size_t)G_ * S.n_u * 32 * w);
    const size_t ns = (size_t)G_ * 32;
    status.ensure(ns * 4); iters.ensure(ns * 4); sing.ensure(ns * 4); piv.ensure(ns * 4);
    maxmis.ensure(ns * 8);
    maxacc.ensure(ns * 8);
    if (want_hist) hist.ensure(ns * std::max(max_iter_, 1) * 8);
    gact.ensure((size_t)G_ * 4); nactive.ensure(16); err.ensure(16);
    o_slot.ensure(ns * 16); o_bf.ensure(ns * 4); o_bt.ensure(ns * 4);
    o_dre.ensure(ns * 32); o_dim.ensure(ns * 32);
    G = G_; prec = prec_; max_iter = max_iter_;
  }

  BatchDev view(bool want_hist, bool outage, double tol, double piv_tol) {
    BatchDev D{};
    D.G = G; D.max_iter = max_iter; D.tol = tol;
    D.vm = vm.as<double>(); D.va = va.as<double>(); D.e = e.as<double>(); D.f = f.as<double>();
    D.psp = psp.as<double>(); D.qsp = qsp.as<double>();
    D.cth = cth.as<double>(); D.sth = sth.as<double>();
    D.eT = eT.p; D.fT = fT.p; D.ivT = ivT.p; D.pT = pT.p; D.qT = qT.p;
    D.jbuf = jbuf.p; D.lu = lu.p; D.off = off.p; D.rhs = rhs.p; D.sol = sol.p;
    D.status = status.as<int32_t>(); D.iters = iters.as<int32_t>(); D.sing = sing.as<int32_t>();
    D.piv_flag = piv.as<int32_t>(); D.maxmis = maxmis.as<double>();
    D.maxacc = maxacc.as<unsigned long long>();
    D.hist = want_hist ? hist.as<double>() : nullptr;
    D.gact = gact.as<int32_t>(); D.nactive = nactive.as<int32_t>();
    D.o_slot = outage ? o_slot.as<int32_t>() : nullptr;
    D.o_bf = outage ? o_bf.as<int32_t>() : nullptr;
    D.o_bt = outage ? o_bt.as<int32_t>() : nullptr;
    D.o_dre = outage ? o_dre.as<double>() : nullptr;
    D.o_dim = outage ? o_dim.as<double>() : nullptr;
    D.piv_tol = prec == GOX_PRECISION_MIXED ? (float)piv_tol : 0.0f;
    D.err = err.as<int32_t>() + 1;
    D.itp = nactive.as<int32_t>() + 1;
    return D;
  }
};

static int grid1d(size_t n, int threads = 256) {
  size_t b = (n + threads - 1) / threads;
  return (int)std::min<size_t>(std::max<size_t>(b, 1), 152 * 32);
}

static constexpr int kWarps = 8;  // warps per CTA of the group kernels

// Dynamic shared memory the refactor may use per CTA (of 227 KB).
static constexpr size_t kRefactorSmem = 225 * 1024;

// How the default refactor plan ends its levels: 1 per-warp progress flags,
// 0 CTA barriers (gox_set_refactor_sync).
static std::atomic<int> g_refactor_sync{0};
// Narrowest refactor level / backward phase the default plan gives the wide
// kernels (0: none; gox_set_refactor_wide).
static std::atomic<int> g_refactor_wide{0};

// Compiles the refactor streams of a schedule for both precisions.
static void make_streams(const Schedule& sc, Stream& s32, Stream& s64) {
  std::string why;
  const int sync = g_refactor_sync.load(), wide = g_refactor_wide.load();
  if (!choose_stream(sc, 4, kRefactorSmem, s32, why, sync, wide))
    throw std::runtime_error("refactor schedule (FP32): " + why);
  if (!choose_stream(sc, 8, kRefactorSmem, s64, why, sync, wide))
    throw std::runtime_error("refactor schedule (FP64): " + why);
  // every stream runs once through the checking host interpreter before a
  // GPU sees it (indices, copies waited for, no cross-warp conflicts)
  std::vector<double> lu(sc.n_slots, 1.0), rhs(sc.n_u, 0.0), X;
  bool sing = false;
  for (const Stream* s : {&s32, &s64}) {
    std::fill(lu.begin(), lu.end(), 1.0);
    const std::string e = run_stream_host(sc, *s, lu, rhs, X, sing);
    if (!e.empty()) throw std::runtime_error("refactor stream check: " + e);
  }
}

struct Timing {
  bool on = false;
  double iters = 0, total = 0, k1 = 0, k2 = 0, k3 = 0, k4 = 0;
};

// Launches one NR iteration's kernels for precision T.
template <typename T>
struct Iter {
  // K5 + K1: update, injections / mismatch, decision.  Returns launches.
  static int mismatch(const SchedDev& S, const BatchDev& D, int it, int mode, bool outage,
                      cudaStream_t st) {
    constexpr int BPW = 4;
    dim3 gu((S.n_bus + 7) / 8, D.G);
    k_update<T><<<gu, 256, 0, st>>>(S, D, it, mode);
    if (mode == 0) {
      dim3 gi((S.n_bus + 8 * BPW - 1) / (8 * BPW), D.G);
      // ZIP terms and outages are compiled in only where a batch has them
      if (S.zip) {
        if (outage) k_inject<T, true, BPW, true><<<gi, 256, 0, st>>>(S, D, it);
        else k_inject<T, false, BPW, true><<<gi, 256, 0, st>>>(S, D, it);
      } else {
        if (outage) k_inject<T, true, BPW, false><<<gi, 256, 0, st>>>(S, D, it);
        else k_inject<T, false, BPW, false><<<gi, 256, 0, st>>>(S, D, it);
      }
    }
    k_decide<<<D.G, 32, 0, st>>>(D, it, mode);
    return mode == 0 ? 3 : 2;
  }
  static void fill(const SchedDev& S, const BatchDev& D, bool outage, cudaStream_t st) {
    const int per_warp = 8;  // tasks per warp
    const int tw = (S.n_ftask + per_warp - 1) / per_warp;
    const int warps = tw + (S.n_fzero + 31) / 32;
    dim3 grid((warps + kWarps - 1) / kWarps, D.G), block(32 * kWarps);
    if (outage) k_fill<T, true><<<grid, block, 0, st>>>(S, D, tw, per_warp);
    else k_fill<T, false><<<grid, block, 0, st>>>(S, D, tw, per_warp);
  }
  static void refactor(const DevSchedule& ds, const BatchDev& D, cudaStream_t st) {
    const int i = sizeof(T) == 4 ? 0 : 1;
    refactor_with(ds, ds.st[i], ds.st_nw[i], ds.st_smem[i], ds.st_wl[i], ds.st_wp[i], ds.st_wr[i], D,
                  D.G, st);
  }
  // the refactor with a given plan's stream over the first `groups` groups:
  // the wide kernels' levels (one launch each), the stream kernel, the wide
  // kernels' backward phases (one launch each)
  static void refactor_with(const DevSchedule& ds, const StreamDev& P, int nw, size_t smem, int wl,
                            int wp, int wr, const BatchDev& D, int groups, cudaStream_t st) {
    wide_pre(ds, wl, wr, D, groups, st);
    stream_kernel(P, nw, smem, ds.d, D, groups, st);
    wide_post(ds, wp, D, groups, st);
  }
  // the wide kernels' refactor levels (before the stream kernel) and their
  // backward-substitution levels (after it)
  static void wide_pre(const DevSchedule& ds, int wl, int wr, const BatchDev& D, int groups,
                       cudaStream_t st) {
    for (int L = 0; L < wl; L++) {
      const long long tasks = (long long)(ds.lev_ptr_h[L + 1] - ds.lev_ptr_h[L]) * groups;
      const unsigned blocks = (unsigned)((tasks + kWideWarps - 1) / kWideWarps);
      wide_attr();
      k_refactor_wide<T><<<blocks, 32 * kWideWarps, wide_smem(wr), st>>>(ds.d, D, L, groups, wr);
    }
  }
  // shared memory of a wide-kernel CTA whose warps stage `rows` rows
  static size_t wide_smem(int rows) { return (size_t)kWideWarps * rows * 32 * sizeof(T); }
  static void wide_post(const DevSchedule& ds, int wp, const BatchDev& D, int groups,
                        cudaStream_t st) {
    for (int L = wp - 1; L >= 0; L--) {
      const long long tasks = (long long)(ds.lev_ptr_h[L + 1] - ds.lev_ptr_h[L]) * groups;
      const unsigned blocks = (unsigned)((tasks + kWideWarps - 1) / kWideWarps);
      k_solve_wide<T><<<blocks, 32 * kWideWarps, 0, st>>>(ds.d, D, L, groups);
    }
  }
  static constexpr size_t kWideSmem = (size_t)kWideWarps * kWideCap * 32 * sizeof(T);
  static void wide_attr() {
    static std::once_flag once[64];
    int dev = 0;
    GOX_CK(cudaGetDevice(&dev));
    std::call_once(once[dev & 63], [] {
      GOX_CK(cudaFuncSetAttribute(k_refactor_wide<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kWideSmem));
    });
  }
  static void stream_kernel(const StreamDev& P, int nw, size_t smem, const SchedDev& S,
                            const BatchDev& D, int groups, cudaStream_t st) {
    // the budget every plan fits in, set once per device (the same value for
    // every plan; setting an attribute per launch would put a driver call
    // between concurrent solves' launches)
    static std::once_flag once[64];
    int dev = 0;
    GOX_CK(cudaGetDevice(&dev));
    std::call_once(once[dev & 63], [] {
      GOX_CK(cudaFuncSetAttribute(k_refactor<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kRefactorSmem));
    });
    k_refactor<T><<<groups, 32 * nw, smem, st>>>(P, S, D);
  }
  static void solve(const SchedDev& S, const BatchDev& D, cudaStream_t st) {
    k_solve<T><<<D.G, 32 * kWarps, 0, st>>>(S, D);
  }
  // the substitutions the refactor's stream did not run (none when it ran
  // the backward substitution too); returns the launches
  static int solve_rest(const DevSchedule& ds, const BatchDev& D, cudaStream_t st) {
    if (ds.st_bwd[sizeof(T) == 4 ? 0 : 1]) return 0;
    solve(ds.d, D, st);
    return 1;
  }
};

}  // namespace gox

using namespace gox;

// ---------------------------------------------------------------------------
// opaque handles

struct IoStage {
  DevMem p, q, vm, va, ovm, ova, it, st, mm, h, sl, dre, dim, pb, qb, sc;
  std::vector<DevMem*> all() {
    return {&p, &q, &vm, &va, &ovm, &ova, &it, &st, &mm, &h, &sl, &dre, &dim, &pb, &qb, &sc};
  }
  size_t bytes() {
    size_t b = 0;
    for (DevMem* m : all()) b += m->bytes;
    return b;
  }
  void release() {
    for (DevMem* m : all()) m->release();
  }
};

// The linear initial guess system of a topology (src/network.rs:627-678),
// built on first use: its pattern, first factor, streams and device buffers.
struct GuessSys {
  bool built = false, usable = false;
  int m = 0, n2 = 0;
  std::vector<int32_t> pq_bus;
  Csc csc;
  Symbolic sym;
  Numeric num;
  Schedule sc;
  Stream s32, s64;
  DevSchedule dsched;
  DevMem yp, yi, yre, yim, rec, rhs_ptr, rhs_ej, pqb, pinv, qinv;
  DevMem lu, off, rhs, sol, sing, piv, gact, err, gvm, gva;
  GuessDev d{};
};

// Staging of the mixed path's FP64 re-solves (rows of the flagged scenarios)
struct FallbackBufs {
  DevMem idx, p, q, vm, va, sl, dr, di, ovm, ova, it, st, mm, hi;
};

// The partial-pivoting factorization of the FP64 re-solves (gox_pivot.cuh):
// each factor column's A entries with their BTF-permuted rows and fill-image
// locations, the right-hand-side positions, and the per-CTA scratch
// (built on first use)
struct PivotPlan {
  bool built = false;
  DevMem R, cp, ci, csrc, rhs_pos, scratch;
  PivotDev d{};
  int max_ctas = 0;
};

// A Newton loop captured as a CUDA graph (conditional while / if nodes),
// keyed by every value its launches bake in
struct LoopGraph {
  std::vector<unsigned char> key;
  cudaGraphExec_t exec = nullptr;
  int uses = 0;
  // a configuration whose host-driven solve re-packed its running scenarios
  // stays on the host-driven loop, where re-packing can run
  bool packs = false;
};

struct gox_topo {
  int n_bus = 0;
  std::vector<int32_t> yp, yi, bus_type;
  std::vector<double> yre, yim;
  JacPattern jac;
  Csc csc;
  Symbolic sym;
  bool factored = false, uploaded = false;
  Numeric num;
  Schedule sc;
  Stream s32, s64;
  DevSchedule dsched;
  DevBatch batch;
  // re-packing: the smaller batch the running scenarios move to, and their
  // scenario indices in the batch
  DevBatch pack;
  DevMem pack_from;
  int64_t repacks = 0;
  Timing timing;
  int64_t launches = 0;
  int device = 0;
  // the refactor plans of the persistent many-topology kernel, per precision
  // (at most 8 warps, no wide split: its CTA runs every phase of a group's
  // Newton loop with the mismatch kernels' 8 warps); built on first use
  struct PersistPlan {
    bool built = false;
    Stream s;
    DevMem words, c0, nc;
    StreamDev d{};
    int nw = 0;
    size_t smem = 0;
  } persist[2];
  // device staging of gox_batch_solve's host arrays (grow-only)
  IoStage io;
  // mixed path: pivot-ratio threshold |u_kk| < piv_tol * max|L(:, k)| that
  // sends a scenario to FP64, and how many the last batch sent
  double piv_tol = 1e-6;
  int64_t fallbacks = 0;
  // start point: 0 as given, 1 the linear initial guess from it
  int guess_mode = 0;
  GuessSys guess;
  // ZIP terms of the effective injection ([4][n]; empty: constant power only)
  std::vector<double> zip;
  DevMem dzip;
  double eff(int part, int i, double s, double vm) const {
    if (zip.empty()) return s;
    s += zip[(size_t)part * n_bus + i] * vm * vm;
    s += zip[(size_t)(2 + part) * n_bus + i] * vm;
    return s;
  }
  // Q-limit enforcement: this topology with PV buses switched to PQ, keyed by
  // the sorted switched buses (owned; built on first use)
  std::vector<std::pair<std::vector<int32_t>, gox_topo*>> variants;
  // bridges of the Y-bus graph and the components without each bridge that
  // an outage has removed (built on first use)
  bool bridges_found = false;
  std::vector<std::pair<int, int>> bridges;
  std::map<std::pair<int, int>, std::vector<int32_t>> splits;
  std::vector<int32_t> base_label;  // components of the graph as registered
  // captured Newton loops (a few keys, oldest replaced) and how many solves used one
  std::vector<LoopGraph> loop_graphs;
  int32_t* h_nactive = nullptr;  // pinned
  FallbackBufs fb;
  // FP64 re-solves of flagged mixed scenarios factor each Jacobian with
  // threshold partial pivoting (set only during those re-solves)
  PivotPlan pplan;
  bool pivot_pass = false;
  // refactor plan chosen by the autotuner, per precision (FP32, FP64)
  bool tune_cache_only = false;  // variants: a cached plan or the default, never timed
  struct Tuning {
    bool done = false;
    int source = 0;  // 0 the default (most warps), 1 measured here, 2 from the cache
    std::vector<std::array<double, 7>> table;  // timed candidates: warps, chunk words, ring rows, ms,
                                               // sync, wide levels, wide phases
  } tune[2];
  // split solves: the parts a large batch is solved in (0: by batch size),
  // and the next instance of this topology (same pivot order, own device
  // buffers and stream) that solves the next part concurrently
  int split_parts = 0;
  std::unique_ptr<gox_topo> twin;
  cudaStream_t own_stream = nullptr;
  bool graphs_off = false;   // a capture failed: the host-driven loop only
  bool graphs_wanted = true;  // gox_topo_set_graph
  int64_t graph_solves = 0;
  ~gox_topo() {
    twin.reset();
    if (own_stream) cudaStreamDestroy(own_stream);
    if (h_nactive) cudaFreeHost(h_nactive);
    for (auto& v : variants) delete v.second;
    for (auto& lg : loop_graphs)
      if (lg.exec) cudaGraphExecDestroy(lg.exec);
  }
};

struct gox_ls {
  int n = 0;
  std::vector<int32_t> rows, cols;
  Csc csc;
  Symbolic sym;
  Numeric num;
  Schedule sc;
  Stream s32, s64;
  DevSchedule dsched;
  DevMem jbuf, lu, off, rhs, sol, sing, piv, gact, status;
  std::vector<double> packed, hostbuf;
};

static int guard_impl(const std::function<int()>& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    return GOX_E_OUT_OF_MEMORY;
  } catch (const CudaError& e) {
    std::fprintf(stderr, "gridoxide_gb300: %s\n", e.what());
    return GOX_E_CUDA;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "gridoxide_gb300: %s\n", e.what());
    return GOX_E_INVALID;
  }
}

// The calling thread's stream for the host-array entry points: created once
// per thread (and device), so that concurrent callers keep distinct streams
// (and hardware queues) instead of a new stream per call
static cudaStream_t thread_stream() {
  struct ThreadStream {
    cudaStream_t s = nullptr;
    int dev = -1;
    ~ThreadStream() {
      if (s) cudaStreamDestroy(s);
    }
  };
  thread_local ThreadStream ts;
  int dev = 0;
  GOX_CK(cudaGetDevice(&dev));
  static std::once_flag pool_once[64];
  std::call_once(pool_once[dev & 63], [dev] {
    // stream-ordered frees keep their memory in the device's pool for the
    // next allocation instead of returning it at every synchronization
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  });
  if (!ts.s || ts.dev != dev) {
    if (ts.s) cudaStreamDestroy(ts.s);
    ts.s = nullptr;
    GOX_CK(cudaStreamCreateWithFlags(&ts.s, cudaStreamNonBlocking));
    ts.dev = dev;
  }
  return ts.s;
}

static int require_device() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return GOX_E_NO_DEVICE;
  }
  return GOX_OK;
}

// Fixes the topology's pivot order from the first scenario whose Jacobian
// at its start point is needed and factors (the first Jacobian a
// PersistentSolver sees, src/solver.rs:711-713).  Returns the scenario index
// used, or -1 when every scenario already meets tol at its start point.
static int fix_pivots(gox_topo* t, int B, const double* p_spec, const double* q_spec,
                      const double* vm0, const double* va0, int v_stride, const int32_t* o_slot,
                      const double* o_dre, const double* o_dim, double tol,
                      std::vector<int>& first_singular) {
  const int n = t->n_bus, nu = t->jac.n_u;
  std::vector<double> p(n), q(n), vals(t->jac.nnz()), yre, yim, packed(t->csc.nnz());
  for (int s = 0; s < B; s++) {
    const double* vm = vm0 + (size_t)s * v_stride;
    const double* va = va0 + (size_t)s * v_stride;
    yre = t->yre;
    yim = t->yim;
    if (o_slot && o_slot[4 * s] >= 0)
      for (int c = 0; c < 4; c++) {
        int sl = o_slot[4 * s + c];
        if (sl < 0 || sl >= (int)yre.size()) throw std::runtime_error("bad outage slot");
        yre[sl] += o_dre[4 * s + c];
        yim[sl] += o_dim[4 * s + c];
      }
    host_injections(n, t->yp.data(), t->yi.data(), yre.data(), yim.data(), vm, va, p.data(),
                    q.data());
    double mx = 0.0;
    for (int a = 0; a < t->jac.n_ang; a++) {
      int i = t->jac.ns_idx[a];
      mx = std::fmax(mx, std::fabs(t->eff(0, i, p_spec[(size_t)s * n + i], vm[i]) - p[i]));
    }
    for (int a = 0; a < t->jac.n_pq; a++) {
      int i = t->jac.pq_idx[a];
      mx = std::fmax(mx, std::fabs(t->eff(1, i, q_spec[(size_t)s * n + i], vm[i]) - q[i]));
    }
    if (mx < tol) continue;
    host_jac_fill(t->jac, yre.data(), yim.data(), vm, va, p.data(), q.data(), vals.data());
    std::fill(packed.begin(), packed.end(), 0.0);
    for (int e = 0; e < t->jac.nnz(); e++) packed[t->csc.slot_of[e]] += vals[e];
    Numeric N;
    if (klu_factor(t->csc, packed.data(), t->sym, 0.001, N) == 0) {
      t->num = std::move(N);
      build_schedule(&t->jac, t->csc, t->sym, t->num, t->sc);
      make_streams(t->sc, t->s32, t->s64);
      t->factored = true;
      t->uploaded = false;
      (void)nu;
      return s;
    }
    first_singular.push_back(s);
  }
  return -1;
}

static constexpr int kGraphMinGroups = 64;  // batches of >= 2,048 scenarios

// The sink (node without dependents) of a graph captured from one stream
static cudaGraphNode_t graph_sink(cudaGraph_t g) {
  size_t n = 0;
  GOX_CK(cudaGraphGetNodes(g, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  GOX_CK(cudaGraphGetNodes(g, nodes.data(), &n));
  for (cudaGraphNode_t v : nodes) {
    size_t m = 0;
    GOX_CK(cudaGraphNodeGetDependentNodes(v, nullptr, nullptr, &m));
    if (m == 0) return v;
  }
  throw std::runtime_error("captured graph without a sink");
}

// Adds a conditional node of `type` on `handle` after `dep` (or at the root)
// and returns its body graph
static cudaGraph_t add_conditional(cudaGraph_t g, cudaGraphNode_t* dep, cudaGraphConditionalHandle h,
                                   cudaGraphConditionalNodeType type, cudaGraphNode_t* out) {
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = type;
  np.conditional.size = 1;
  GOX_CK(cudaGraphAddNode(out, g, dep, nullptr, dep ? 1 : 0, &np));
  return np.conditional.phGraph_out[0];
}

// The whole Newton loop as one graph: it = 0; while (running) { mismatch;
// decision; if (running) { fill; refactor; solves } }; if (budget spent)
// { final mismatch }.  Kernels read the iteration from D.itp.
template <typename T>
static cudaGraphExec_t build_loop_graph(gox_topo* t, const BatchDev& D, int max_iter, bool outage,
                                        cudaStream_t st) {
  const SchedDev& S = t->dsched.d;
  cudaGraph_t g = nullptr;
  GOX_CK(cudaGraphCreate(&g, 0));
  struct GraphGuard {
    cudaGraph_t g;
    ~GraphGuard() { cudaGraphDestroy(g); }
  } gg{g};
  cudaGraphConditionalHandle hw, hif, hmax;
  GOX_CK(cudaGraphConditionalHandleCreate(&hw, g, 1, cudaGraphCondAssignDefault));
  GOX_CK(cudaGraphConditionalHandleCreate(&hif, g, 0, cudaGraphCondAssignDefault));
  GOX_CK(cudaGraphConditionalHandleCreate(&hmax, g, 0, cudaGraphCondAssignDefault));
  cudaGraphNode_t n0, nw, nif, nmax;
  cudaMemsetParams mp{};
  mp.dst = D.itp; mp.value = 0; mp.elementSize = 4; mp.width = 1; mp.height = 1;
  GOX_CK(cudaGraphAddMemsetNode(&n0, g, nullptr, 0, &mp));
  cudaGraph_t body = add_conditional(g, &n0, hw, cudaGraphCondTypeWhile, &nw);
  cudaGraph_t cap = nullptr;
  GOX_CK(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  GOX_CK(cudaMemsetAsync(D.nactive, 0, sizeof(int32_t), st));
  Iter<T>::mismatch(S, D, -1, 0, outage, st);
  k_cond<<<1, 1, 0, st>>>(D.nactive, D.itp, max_iter, hw, hif, hmax);
  GOX_CK(cudaStreamEndCapture(st, &cap));
  cudaGraphNode_t sink = graph_sink(body);
  cudaGraph_t ifb = add_conditional(body, &sink, hif, cudaGraphCondTypeIf, &nif);
  GOX_CK(cudaStreamBeginCaptureToGraph(st, ifb, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  Iter<T>::fill(S, D, outage, st);
  Iter<T>::refactor(t->dsched, D, st);
  Iter<T>::solve_rest(t->dsched, D, st);
  GOX_CK(cudaStreamEndCapture(st, &cap));
  cudaGraph_t mb = add_conditional(g, &nw, hmax, cudaGraphCondTypeIf, &nmax);
  GOX_CK(cudaStreamBeginCaptureToGraph(st, mb, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  Iter<T>::mismatch(S, D, -1, 1, outage, st);
  GOX_CK(cudaStreamEndCapture(st, &cap));
  cudaGraphExec_t ex = nullptr;
  GOX_CK(cudaGraphInstantiate(&ex, g, 0));
  return ex;
}

// Runs the loop from a cached graph when this exact configuration was seen
// before (the first sighting runs the host loop and records the key);
// false: run the host loop.
// Everything a captured loop bakes in: precision (first 4 bytes), budget,
// outage use, buffers, schedule and the refactor stream.
template <typename T>
static std::vector<unsigned char> loop_key(const gox_topo* t, const BatchDev& D, int max_iter,
                                           bool outage) {
  std::vector<unsigned char> key;
  auto put = [&](const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    key.insert(key.end(), c, c + n);
  };
  const int prec = (int)sizeof(T), i = sizeof(T) == 4 ? 0 : 1;
  const unsigned char o = outage ? 1 : 0;
  put(&prec, sizeof prec); put(&max_iter, sizeof max_iter); put(&o, 1);
  put(&D, sizeof D); put(&t->dsched.d, sizeof(SchedDev));
  put(&t->dsched.st[i], sizeof(StreamDev)); put(&t->dsched.st_nw[i], sizeof(int));
  put(&t->dsched.st_smem[i], sizeof(size_t)); put(&t->dsched.st_bwd[i], sizeof(bool));
  put(&t->dsched.st_wl[i], sizeof(int)); put(&t->dsched.st_wp[i], sizeof(int));
  put(&t->dsched.st_wr[i], sizeof(int));
  return key;
}

// A configuration seen once: its next solve captures and runs the graph.
static void remember_loop(gox_topo* t, const std::vector<unsigned char>& key) {
  for (auto& x : t->loop_graphs)
    if (x.key == key) return;
  if (t->loop_graphs.size() >= 4) {
    if (t->loop_graphs.front().exec) cudaGraphExecDestroy(t->loop_graphs.front().exec);
    t->loop_graphs.erase(t->loop_graphs.begin());
  }
  t->loop_graphs.push_back(LoopGraph{key, nullptr, 1});
}

template <typename T>
static bool run_loop_graph(gox_topo* t, const BatchDev& D, int max_iter, bool outage,
                           cudaStream_t st) {
  // small batches stay on the host-driven loop: measured, their graphs ran
  // slower when many topologies solve concurrently from several threads
  if (t->graphs_off || !t->graphs_wanted || D.G < kGraphMinGroups) return false;
  const std::vector<unsigned char> key = loop_key<T>(t, D, max_iter, outage);
  LoopGraph* lg = nullptr;
  for (auto& x : t->loop_graphs)
    if (x.key == key) lg = &x;
  if (!lg) {
    remember_loop(t, key);
    return false;
  }
  if (lg->packs) return false;
  if (!lg->exec) {
    try {
      lg->exec = build_loop_graph<T>(t, D, max_iter, outage, st);
    } catch (...) {
      // a capture that failed leaves the stream capturing: end it, and keep
      // this topology on the host loop
      cudaGraph_t junk = nullptr;
      cudaStreamCaptureStatus cs;
      if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
        cudaStreamEndCapture(st, &junk);
      if (junk) cudaGraphDestroy(junk);
      cudaGetLastError();
      t->graphs_off = true;
      return false;
    }
  }
  lg->uses++;
  GOX_CK(cudaGraphLaunch(lg->exec, st));
  t->graph_solves++;
  return true;
}

// Scratch bound of a scenario's pivoting factor: the static pattern three
// times over plus four entries per column (partial pivoting changes the
// pattern; a factor that outgrows this marks its scenario singular).
static void pivot_plan_build(gox_topo* t) {
  PivotPlan& PP = t->pplan;
  const Schedule& sc = t->sc;
  const Symbolic& S = t->sym;
  const Csc& A = t->csc;
  const int n = sc.n_u;
  std::vector<int32_t> psinv(n), a_of_csc(A.nnz(), -1), cp(n + 1, 0), ci, csrc, rhs_pos(n);
  for (int i = 0; i < n; i++) psinv[S.P[i]] = i;
  for (int a = 0; a < sc.n_a; a++) a_of_csc[sc.a_csc[a]] = a;
  for (int k = 0; k < n; k++) {
    const int oc = S.Q[k];
    for (int p = A.p[oc]; p < A.p[oc + 1]; p++) {
      const int a = a_of_csc[p];
      if (a < 0) throw std::runtime_error("pivot plan: an A entry without a fill destination");
      ci.push_back(psinv[A.i[p]]);
      csrc.push_back(sc.a_dst[a] >= 0 ? sc.c_base[k] + sc.a_dst[a] : sc.a_dst[a]);
    }
    cp[k + 1] = (int)ci.size();
  }
  for (int i = 0; i < n; i++) rhs_pos[i] = t->num.Pinv[S.P[i]];
  upload(PP.R, S.R);
  upload(PP.cp, cp);
  upload(PP.ci, ci);
  upload(PP.csrc, csrc);
  upload(PP.rhs_pos, rhs_pos);
  PivotDev& d = PP.d;
  d.n = n;
  d.nblocks = S.nblocks;
  d.n_slots = sc.n_slots;
  d.n_off = sc.n_off;
  const int nlu = (int)(t->num.Li.size() + t->num.Ui.size());
  d.lcap = 3 * nlu + 4 * n;
  d.ucap = 3 * nlu + 4 * n;
  d.ocap = std::max(sc.n_off, 1);
  d.R = PP.R.as<int32_t>();
  d.cp = PP.cp.as<int32_t>();
  d.ci = PP.ci.as<int32_t>();
  d.csrc = PP.csrc.as<int32_t>();
  d.rhs_pos = PP.rhs_pos.as<int32_t>();
  d.tol = 0.001;  // KLU's default pivot tolerance (klu_defaults.c), as KluNative
  d.stride = pivot_stride(n, d.lcap, d.ucap, d.ocap);
  // as many CTAs as 4 GB of scratch hold (at least one per SM)
  PP.max_ctas = (int)std::max<size_t>(152, ((size_t)4 << 30) / d.stride);
  PP.built = true;
}

// The pivoting factorization + solve of every running scenario of the batch
// (FP64 buffers), in place of the static refactor and substitutions.
static void pivot_run(gox_topo* t, BatchDev& D, cudaStream_t st) {
  PivotPlan& PP = t->pplan;
  if (!PP.built) pivot_plan_build(t);
  const int ctas = std::min(D.G * 32, PP.max_ctas);
  PP.scratch.ensure((size_t)ctas * PP.d.stride);
  PP.d.scratch = PP.scratch.as<unsigned char>();
  k_factor_pivot<<<ctas, 32, 0, st>>>(PP.d, D);
}

// ---------------------------------------------------------------------------
// Refactor autotuner.  The plan of a topology's refactor streams (warps per
// CTA, stream-chunk words, hence ring rows) is chosen by timing the
// candidate plans on the first batch the topology solves in a precision:
// after that batch's first Jacobian fill, each candidate's stream (compiled
// on the host and checked by the host interpreter first) refactors the
// first min(G, 152) groups of the image, twice, timed with CUDA events on
// the solve stream; the fastest is kept.  The choice is cached per process
// (and in the file $GOX_TUNE_CACHE, when set) under (precision, bus-count
// bucket of half an octave, fill nnz(L+U) / nnz(J) in tenths, batch size
// in groups: 1, 2-8, 9-38, 39-152, more); a topology with a cached key
// compiles that plan only.  gox_set_autotune(0) keeps the default plan
// (the most warps that fit).

static std::mutex g_tune_mu;
// key -> {warps, chunk words, sync, wide split (0 none, else its narrowest level width)}
static std::map<std::array<int, 4>, std::array<int, 4>> g_tune;
static bool g_tune_loaded = false;
static std::atomic<int> g_autotune{1};

static std::array<int, 4> tune_key(const gox_topo* t, int prec, int groups) {
  const double fill = (double)(t->num.Li.size() + t->num.Ui.size() + t->num.Pnum.size()) /
                      (double)std::max(1, t->jac.nnz());
  const int gb = groups <= 1 ? 0 : groups <= 8 ? 1 : groups <= 38 ? 2 : groups <= 152 ? 3 : 4;
  return {prec, (int)std::lround(2.0 * std::log2((double)std::max(2, t->n_bus))),
          (int)std::lround(10.0 * fill), gb};
}

static void tune_cache_load() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* path = std::getenv("GOX_TUNE_CACHE");
  if (!path || !*path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  int a, b, c, d, nw, cw, sy, wd;
  while (std::fscanf(f, "gox-tune-3 %d %d %d %d %d %d %d %d\n", &a, &b, &c, &d, &nw, &cw, &sy, &wd) == 8)
    g_tune[{a, b, c, d}] = {nw, cw, sy, wd};
  std::fclose(f);
}

static void tune_cache_store(const std::array<int, 4>& k, const StreamPlan& p) {
  const int nw = p.nw, cw = p.chunk_words, sy = p.sync, wd = p.wide_levels > 0 ? p.wide_min : 0;
  g_tune[k] = {nw, cw, sy, wd};
  const char* path = std::getenv("GOX_TUNE_CACHE");
  if (!path || !*path) return;
  if (FILE* f = std::fopen(path, "a")) {
    std::fprintf(f, "gox-tune-3 %d %d %d %d %d %d %d %d\n", k[0], k[1], k[2], k[3], nw, cw, sy, wd);
    std::fclose(f);
  }
}

// Compiles a plan's stream and runs it once through the checking host
// interpreter (as make_streams does for the default plan).
static bool compile_checked(const Schedule& sc, const StreamPlan& p, Stream& out) {
  std::string why;
  if (!build_plan(sc, p, out, why)) return false;
  std::vector<double> lu(sc.n_slots, 1.0), rhs(sc.n_u, 0.0), X;
  bool sing = false;
  return run_stream_host(sc, out, lu, rhs, X, sing).empty();
}

// Installs a precision's stream on the topology (and its split twin); the
// captured Newton loops hold the old stream's device pointers: dropped.
static void drop_loops(gox_topo* t, int i) {
  const int prec = i == 0 ? 4 : 8;
  std::vector<LoopGraph> keep;
  for (auto& lg : t->loop_graphs) {
    int kp = 0;
    std::memcpy(&kp, lg.key.data(), sizeof kp);
    if (kp == prec) {
      if (lg.exec) cudaGraphExecDestroy(lg.exec);
    } else {
      keep.push_back(std::move(lg));
    }
  }
  t->loop_graphs = std::move(keep);
}

static void install_stream(gox_topo* t, int i, Stream&& s) {
  (i == 0 ? t->s32 : t->s64) = std::move(s);
  t->dsched.load_streams(t->s32, t->s64);
  drop_loops(t, i);
  // the split solves' twins (a chain: the twin of part k solves part k + 1)
  for (gox_topo* tw = t->twin.get(); tw; tw = tw->twin.get()) {
    tw->s32 = t->s32;
    tw->s64 = t->s64;
    if (tw->uploaded) tw->dsched.load_streams(tw->s32, tw->s64);
    drop_loops(tw, i);
  }
}

template <typename T>
static void autotune(gox_topo* t, const BatchDev& D, cudaStream_t st) {
  const int i = sizeof(T) == 4 ? 0 : 1;
  gox_topo::Tuning& TU = t->tune[i];
  TU.done = true;
  if (!g_autotune.load()) return;
  const Schedule& sc = t->sc;
  const int elem = (int)sizeof(T);
  const std::array<int, 4> key = tune_key(t, i, D.G);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_cache_load();
    auto it = g_tune.find(key);
    if (it == g_tune.end() && t->tune_cache_only) return;
    if (it != g_tune.end()) {
      const Stream& cur = i == 0 ? t->s32 : t->s64;
      auto same = [&](const StreamPlan& p) {
        return p.nw == it->second[0] && p.chunk_words == it->second[1] && p.sync == it->second[2] &&
               (p.wide_levels > 0 ? p.wide_min : 0) == it->second[3];
      };
      if (same(cur.plan)) {
        TU.source = 2;
        return;
      }
      for (const StreamPlan& p : candidate_plans(sc, elem, kRefactorSmem))
        if (same(p)) {
          Stream s;
          if (compile_checked(sc, p, s)) {
            install_stream(t, i, std::move(s));
            TU.source = 2;
            return;
          }
          break;
        }
      // the cached plan does not fit this topology (another topology of the
      // same size and fill bucket, e.g. one whose first level can go to the
      // wide kernels): time the candidates, unless timing is not allowed
      if (t->tune_cache_only) return;
    }
  }
  // compile and check every candidate (host threads in parallel)
  std::vector<StreamPlan> cand = candidate_plans(sc, elem, kRefactorSmem);
  std::vector<Stream> built(cand.size());
  std::vector<char> ok(cand.size(), 0);
  {
    std::vector<std::thread> th;
    std::atomic<size_t> next{0};
    const unsigned nt = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    for (unsigned w = 0; w < nt; w++)
      th.emplace_back([&] {
        for (size_t c; (c = next++) < cand.size();) ok[c] = compile_checked(sc, cand[c], built[c]);
      });
    for (auto& x : th) x.join();
  }
  const int Gt = std::min(D.G, 152);
  const size_t img_bytes = (size_t)Gt * sc.n_slots * 32 * sizeof(T);
  DevMem bak, words, c0, nc;
  bak.ensure(img_bytes);
  GOX_CK(cudaMemcpyAsync(bak.p, D.lu, img_bytes, cudaMemcpyDeviceToDevice, st));
  cudaEvent_t e0, e1;
  GOX_CK(cudaEventCreate(&e0));
  GOX_CK(cudaEventCreate(&e1));
  double best_ms = 1e30;
  int best = -1;
  TU.table.clear();
  for (size_t c = 0; c < cand.size(); c++) {
    if (!ok[c]) continue;
    const Stream& s = built[c];
    upload(words, s.words);
    upload(c0, s.chunk0);
    upload(nc, s.nchunks);
    StreamDev P{};
    P.words = words.as<int32_t>();
    P.chunk0 = c0.as<int32_t>();
    P.nchunks = nc.as<int32_t>();
    P.ring_rows = s.plan.ring_rows;
    P.rows_total = ring_total(s.plan);
    P.chunk_words = s.plan.chunk_words;
    P.n_bars = s.n_bars;
    P.sync = s.plan.sync;
    float ms = 0.0f;
    for (int rep = 0; rep < 2; rep++) {
      GOX_CK(cudaMemcpyAsync(D.lu, bak.p, img_bytes, cudaMemcpyDeviceToDevice, st));
      GOX_CK(cudaEventRecord(e0, st));
      Iter<T>::refactor_with(t->dsched, P, s.plan.nw, stream_smem_bytes(s.plan), s.plan.wide_levels,
                             s.plan.wide_phases, s.plan.wide_rows, D, Gt, st);
      GOX_CK(cudaEventRecord(e1, st));
      GOX_CK(cudaEventSynchronize(e1));
      GOX_CK(cudaEventElapsedTime(&ms, e0, e1));
    }
    GOX_CK(cudaGetLastError());
    int32_t herr[2] = {0, 0};
    GOX_CK(cudaMemcpyAsync(herr, D.err - 1, 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    if (herr[1]) {  // a bounded wait gave up under this plan: not a candidate
      const int32_t z[2] = {0, 0};
      GOX_CK(cudaMemcpyAsync(D.err - 1, z, 8, cudaMemcpyHostToDevice, st));
      continue;
    }
    TU.table.push_back({(double)s.plan.nw, (double)s.plan.chunk_words, (double)s.plan.ring_rows,
                        (double)ms, (double)s.plan.sync, (double)s.plan.wide_levels,
                        (double)s.plan.wide_phases});
    if (ms < best_ms) {
      best_ms = ms;
      best = (int)c;
    }
  }
  // the image as the fill left it, for the iteration to go on
  GOX_CK(cudaMemcpyAsync(D.lu, bak.p, img_bytes, cudaMemcpyDeviceToDevice, st));
  GOX_CK(cudaStreamSynchronize(st));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best < 0) return;
  const StreamPlan bestp = cand[best];
  install_stream(t, i, std::move(built[best]));
  TU.source = 1;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  tune_cache_store(key, bestp);
}

// Re-packing of the running scenarios (host-driven loop).  After an
// iteration's decision, when the scenarios still running fit in at most half
// of the groups still active, they move into the first lanes of a smaller
// batch (t->pack) and the remaining iterations run there; at the end their
// results go back to their own lanes.  Every kernel's arithmetic is per
// lane, so a scenario's result is the same in either batch, bit for bit.
// Fewer groups mean fewer mismatch and fill blocks and, when the batch spans
// more than one wave of refactor CTAs, fewer waves.
static constexpr int kPackMinGroups = 16;
static std::atomic<int> g_repack{1};  // gox_set_repack

template <typename T>
static bool repack(gox_topo* t, const BatchDev& D, bool outage, int active_groups,
                   cudaStream_t st, BatchDev& P, int& R, int64_t& launches) {
  const int G = D.G;
  std::vector<int32_t> status((size_t)G * 32);
  GOX_CK(cudaMemcpyAsync(status.data(), D.status, status.size() * 4, cudaMemcpyDeviceToHost, st));
  GOX_CK(cudaStreamSynchronize(st));
  std::vector<int32_t> from;
  for (int s = 0; s < G * 32; s++)
    if (status[s] == ST_RUNNING) from.push_back(s);
  R = (int)from.size();
  const int Gp = (R + 31) / 32;
  if (R == 0 || 2 * Gp > active_groups) return false;
  const SchedDev& S = t->dsched.d;
  const int prec = sizeof(T) == 4 ? GOX_PRECISION_MIXED : GOX_PRECISION_FP64;
  const bool hist = D.hist != nullptr;
  DevBatch& PB = t->pack;
  PB.ensure(S, Gp, prec, D.max_iter, hist);
  P = PB.view(hist, outage, D.tol, 0.0);
  P.piv_tol = D.piv_tol;
  P.err = D.err;  // one error flag for the solve
  upload(t->pack_from, from);
  const int32_t* fr = t->pack_from.as<int32_t>();
  using U8 = unsigned long long;
  using W = typename std::conditional<sizeof(T) == 4, uint32_t, U8>::type;
  const int n = S.n_bus, nu = S.n_u, K = Gp * 32;
  auto rows8 = [&](const double* a, double* b, int rows) {
    k_pack_rows<U8><<<grid1d((size_t)K * rows), 256, 0, st>>>((const U8*)a, (U8*)b, rows, fr, R, Gp);
    launches++;
  };
  auto rowsT = [&](const void* a, void* b, int rows) {
    k_pack_rows<W><<<grid1d((size_t)K * rows), 256, 0, st>>>((const W*)a, (W*)b, rows, fr, R, Gp);
    launches++;
  };
  auto flat4 = [&](const void* a, void* b, int width) {
    k_pack_flat<uint32_t><<<grid1d((size_t)K * width), 256, 0, st>>>((const uint32_t*)a,
                                                                       (uint32_t*)b, width, fr, R, K);
    launches++;
  };
  auto flat8 = [&](const void* a, void* b, int width) {
    k_pack_flat<U8><<<grid1d((size_t)K * width), 256, 0, st>>>((const U8*)a, (U8*)b, width, fr, R, K);
    launches++;
  };
  // the state the rest of this iteration (fill, refactor) and the next ones read
  rows8(D.vm, P.vm, n); rows8(D.va, P.va, n); rows8(D.cth, P.cth, n); rows8(D.sth, P.sth, n);
  rows8(D.psp, P.psp, n); rows8(D.qsp, P.qsp, n);
  rowsT(D.eT, P.eT, n); rowsT(D.fT, P.fT, n); rowsT(D.ivT, P.ivT, n);
  rowsT(D.pT, P.pT, n); rowsT(D.qT, P.qT, n); rowsT(D.rhs, P.rhs, nu);
  flat4(D.status, P.status, 1); flat4(D.iters, P.iters, 1); flat4(D.sing, P.sing, 1);
  flat4(D.piv_flag, P.piv_flag, 1); flat8(D.maxmis, P.maxmis, 1);
  if (hist) flat8(D.hist, P.hist, D.max_iter);
  if (outage) {
    flat4(D.o_slot, PB.o_slot.p, 4); flat4(D.o_bf, PB.o_bf.p, 1); flat4(D.o_bt, PB.o_bt.p, 1);
    flat8(D.o_dre, PB.o_dre.p, 4); flat8(D.o_dim, PB.o_dim.p, 4);
  }
  GOX_CK(cudaMemsetAsync(P.maxacc, 0, (size_t)K * 8, st));
  k_pack_mark<<<(K + 255) / 256, 256, 0, st>>>(P.status, P.gact, R, Gp);
  launches++;
  GOX_CK(cudaGetLastError());
  t->repacks++;
  return true;
}

// The packed scenarios' results back to their lanes of the batch.
template <typename T>
static void unpack(gox_topo* t, const BatchDev& P, const BatchDev& D, int R, cudaStream_t st,
                   int64_t& launches) {
  using U8 = unsigned long long;
  const int n = t->dsched.d.n_bus;
  const int32_t* fr = t->pack_from.as<int32_t>();
  for (auto pr : {std::make_pair(P.vm, D.vm), std::make_pair(P.va, D.va)}) {
    k_unpack_rows<U8><<<grid1d((size_t)R * n), 256, 0, st>>>((const U8*)pr.first, (U8*)pr.second,
                                                             n, fr, R);
    launches++;
  }
  for (auto pr : {std::make_pair(P.status, D.status), std::make_pair(P.iters, D.iters),
                  std::make_pair(P.sing, D.sing), std::make_pair(P.piv_flag, D.piv_flag)}) {
    k_unpack_flat<uint32_t><<<grid1d((size_t)R), 256, 0, st>>>((const uint32_t*)pr.first,
                                                                (uint32_t*)pr.second, 1, fr, R);
    launches++;
  }
  k_unpack_flat<U8><<<grid1d((size_t)R), 256, 0, st>>>((const U8*)P.maxmis, (U8*)D.maxmis, 1, fr, R);
  launches++;
  if (D.hist) {
    k_unpack_flat<U8><<<grid1d((size_t)R * D.max_iter), 256, 0, st>>>(
        (const U8*)P.hist, (U8*)D.hist, D.max_iter, fr, R);
    launches++;
  }
  GOX_CK(cudaGetLastError());
}

template <typename T>
static void run_iterations(gox_topo* t, BatchDev D, int max_iter, bool outage, cudaStream_t st,
                           int32_t* h_nactive) {
  const SchedDev& S = t->dsched.d;
  const bool timing = t->timing.on;
  const bool pivoting = sizeof(T) == 8 && t->pivot_pass;
  if (!timing && !pivoting && run_loop_graph<T>(t, D, max_iter, outage, st)) {
    // launches: per iteration 3 + 1 (decision) and, while running, fill,
    // refactor and the separate solve; the final mismatch when the budget ran out
    int32_t h[2] = {0, 0};
    GOX_CK(cudaMemcpyAsync(h, D.nactive, 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    const int its = h[1], ran_out = (h[0] > 0 && its >= max_iter) ? 1 : 0;
    const int fills = h[0] > 0 ? its : its - 1;
    const int ns = t->dsched.st_bwd[sizeof(T) == 4 ? 0 : 1] ? 0 : 1;
    const int nr = t->dsched.refactor_launches(sizeof(T) == 4 ? 0 : 1);
    t->launches += (int64_t)its * 4 + (int64_t)fills * (1 + nr + ns) + ran_out * 2;
    return;
  }
  // events: per iteration [k1 start, k1 end, k2 end, k3 end, k4 end]; read once at the end
  std::vector<cudaEvent_t> ev;
  auto rec = [&]() {
    if (!timing) return;
    cudaEvent_t e;
    GOX_CK(cudaEventCreate(&e));
    GOX_CK(cudaEventRecord(e, st));
    ev.push_back(e);
  };
  int it = 0;
  bool tuned_now = false;
  std::vector<int> full;  // iterations that ran K2-K4
  const BatchDev D0 = D;   // the batch (D becomes the packed one after a re-pack)
  bool packed = false;
  int R = 0;
  rec();
  for (it = 0; it < max_iter; it++) {
    GOX_CK(cudaMemsetAsync(D.nactive, 0, sizeof(int32_t), st));
    rec();
    t->launches += Iter<T>::mismatch(S, D, it, 0, outage, st);
    rec();
    GOX_CK(cudaMemcpyAsync(h_nactive, D.nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    if (*h_nactive == 0) break;
    if (!packed && !pivoting && it > 0 && *h_nactive >= kPackMinGroups && g_repack.load()) {
      BatchDev P{};
      if (repack<T>(t, D, outage, *h_nactive, st, P, R, t->launches)) {
        D = P;
        packed = true;
      }
    }
    Iter<T>::fill(S, D, outage, st);
    if (!pivoting && !t->tune[sizeof(T) == 4 ? 0 : 1].done) {
      autotune<T>(t, D, st);
      tuned_now = true;
    }
    rec();
    int ns = 0;
    if (pivoting) {
      pivot_run(t, D, st);
      rec();
    } else {
      Iter<T>::refactor(t->dsched, D, st);
      rec();
      ns = Iter<T>::solve_rest(t->dsched, D, st);
    }
    rec();
    t->launches += 1 + t->dsched.refactor_launches(sizeof(T) == 4 ? 0 : 1) + ns;
    GOX_CK(cudaGetLastError());
  }
  if (it == max_iter) t->launches += Iter<T>::mismatch(S, D, max_iter, 1, outage, st);
  if (packed) {
    unpack<T>(t, D, D0, R, st, t->launches);
    // this configuration stays on the host-driven loop
    const std::vector<unsigned char> key = loop_key<T>(t, D0, max_iter, outage);
    remember_loop(t, key);
    for (auto& x : t->loop_graphs)
      if (x.key == key) x.packs = true;
  }
  rec();
  GOX_CK(cudaGetLastError());
  // the plan chosen during this solve changed the loop's key: remember the
  // new configuration, so that the next solve runs it as a graph
  if (tuned_now && !timing && !pivoting && !t->graphs_off && t->graphs_wanted &&
      D0.G >= kGraphMinGroups)
    remember_loop(t, loop_key<T>(t, D0, max_iter, outage));
  if (timing) {
    GOX_CK(cudaEventSynchronize(ev.back()));
    auto el = [&](size_t a, size_t b) {
      float ms = 0;
      GOX_CK(cudaEventElapsedTime(&ms, ev[a], ev[b]));
      return (double)ms;
    };
    Timing& T_ = t->timing;
    T_.iters = it;
    T_.total = el(0, ev.size() - 1);
    T_.k1 = T_.k2 = T_.k3 = T_.k4 = 0;
    size_t i = 1;
    for (int k = 0; k <= it && k < max_iter; k++) {
      if (i + 1 >= ev.size()) break;
      T_.k1 += el(i, i + 1);
      if (i + 4 < ev.size() && k < it) {
        T_.k2 += el(i + 1, i + 2);
        T_.k3 += el(i + 2, i + 3);
        T_.k4 += el(i + 3, i + 4);
        i += 5;
      } else {
        break;
      }
    }
    for (auto e : ev) cudaEventDestroy(e);
  }
}

// Core of both batch entry points: all arrays on the device.
// Builds the guess system from scenario 0's injections (host arrays p0, q0):
// the PQ buses, the 2x2 real blocks of Y' between them, the fixed neighbours
// of each, the first factorization (partial pivoting) and its streams.
static void guess_build(gox_topo* t, const double* p0, const double* q0) {
  GuessSys& G = t->guess;
  G.built = true;
  G.usable = false;
  const int n = t->n_bus;
  std::vector<int32_t> rpos(n, -1);
  G.pq_bus.clear();
  for (int i = 0; i < n; i++)
    if (t->bus_type[i] == 1) {
      rpos[i] = (int)G.pq_bus.size();
      G.pq_bus.push_back(i);
    }
  G.m = (int)G.pq_bus.size();
  G.n2 = 2 * G.m;
  if (G.m == 0) return;
  std::vector<int32_t> rows, cols, rp(1, 0);
  std::vector<int32_t> rec4;  // per triplet {part, Y entry, load bus, 0}
  std::vector<int32_t> ej;
  std::vector<double> vals;
  auto block = [&](int r, int c, int e, int load) {
    const double yr = (e >= 0 ? t->yre[e] : 0.0) + (load >= 0 ? -p0[load] : 0.0);
    const double yi = (e >= 0 ? t->yim[e] : 0.0) + (load >= 0 ? q0[load] : 0.0);
    const int rr[4] = {2 * r, 2 * r, 2 * r + 1, 2 * r + 1}, cc[4] = {2 * c, 2 * c + 1, 2 * c, 2 * c + 1};
    const int part[4] = {0, 1, 2, 0};
    const double v[4] = {yr, -yi, yi, yr};
    for (int k = 0; k < 4; k++) {
      rows.push_back(rr[k]);
      cols.push_back(cc[k]);
      vals.push_back(v[k]);
      rec4.insert(rec4.end(), {part[k], e, load, 0});
    }
  };
  for (int r = 0; r < G.m; r++) {
    const int i = G.pq_bus[r];
    bool diag = false;
    for (int e = t->yp[i]; e < t->yp[i + 1]; e++) {
      const int j = t->yi[e];
      if (j == i) {
        diag = true;
        block(r, r, e, i);
      } else if (rpos[j] >= 0) {
        block(r, rpos[j], e, -1);
      } else {
        ej.insert(ej.end(), {e, j});
      }
    }
    if (!diag) block(r, r, -1, i);
    rp.push_back((int32_t)(ej.size() / 2));
  }
  const int nnz = (int)rows.size();
  G.csc = build_csc(G.n2, nnz, rows.data(), cols.data());
  G.sym = klu_analyze(G.n2, G.csc.p.data(), G.csc.i.data());
  std::vector<double> packed(G.csc.nnz(), 0.0);
  std::vector<int32_t> trip_of(G.csc.nnz(), -1);
  for (int e = 0; e < nnz; e++) {
    packed[G.csc.slot_of[e]] += vals[e];
    trip_of[G.csc.slot_of[e]] = e;
  }
  if (klu_factor(G.csc, packed.data(), G.sym, 0.001, G.num) != 0) return;
  build_schedule(nullptr, G.csc, G.sym, G.num, G.sc);
  make_streams(G.sc, G.s32, G.s64);
  std::vector<int32_t> dummy_p(1, 0), dummy_i;
  std::vector<double> dummy_x;
  G.dsched.load(G.sc, dummy_p, dummy_i, dummy_x, dummy_x);
  G.dsched.load_streams(G.s32, G.s64);
  // value recipe per LU slot, then per off-diagonal entry
  const int ns = G.sc.n_slots, no = G.sc.n_off;
  std::vector<int32_t> rec((size_t)(ns + no) * 4);
  for (int x = 0; x < ns + no; x++) {
    const int a = x < ns ? G.sc.slot_a[x] : G.sc.off_a[x - ns];
    int32_t* r = &rec[(size_t)x * 4];
    if (a < 0) {
      r[0] = -1; r[1] = -1; r[2] = -1; r[3] = 0;
      continue;
    }
    const int tr = trip_of[G.sc.a_csc[a]];
    if (tr < 0) throw std::logic_error("guess system entry without a source");
    for (int k = 0; k < 4; k++) r[k] = rec4[(size_t)tr * 4 + k];
  }
  std::vector<int32_t> pinv(G.n2), qinv(G.n2);
  for (int k = 0; k < G.n2; k++) {
    pinv[G.num.Pnum[k]] = k;
    qinv[G.sym.Q[k]] = k;
  }
  upload(G.yp, t->yp);
  upload(G.yi, t->yi);
  upload(G.yre, t->yre);
  upload(G.yim, t->yim);
  upload(G.rec, rec);
  upload(G.rhs_ptr, rp);
  upload(G.rhs_ej, ej);
  upload(G.pqb, G.pq_bus);
  upload(G.pinv, pinv);
  upload(G.qinv, qinv);
  GuessDev& d = G.d;
  d.n_bus = n; d.m = G.m; d.n2 = G.n2; d.n_slots = ns; d.n_off = no;
  d.yp = G.yp.as<int32_t>(); d.yi = G.yi.as<int32_t>(); d.yre = G.yre.as<double>(); d.yim = G.yim.as<double>();
  d.rec = reinterpret_cast<const int4*>(G.rec.p);
  d.rhs_ptr = G.rhs_ptr.as<int32_t>();
  d.rhs_ej = reinterpret_cast<const int2*>(G.rhs_ej.p);
  d.pq_bus = G.pqb.as<int32_t>();
  d.pinv = G.pinv.as<int32_t>();
  d.qinv = G.qinv.as<int32_t>();
  G.usable = true;
}

// The linear initial guess of B scenarios (device arrays, start voltages
// vm0/va0 with stride v_stride): their start points in G.gvm / G.gva [B][N].
// False when the topology has no PQ bus or its guess system is singular at
// its first factorization (the start points then stay as given).
static bool guess_run(gox_topo* t, int B, const double* p_spec, const double* q_spec,
                      const double* vm0, const double* va0, int v_stride, const int32_t* o_slot,
                      const double* o_dre, const double* o_dim, cudaStream_t st) {
  GuessSys& G = t->guess;
  const int n = t->n_bus;
  if (!G.built) {
    std::vector<double> p0(n), q0(n);
    GOX_CK(cudaMemcpyAsync(p0.data(), p_spec, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(q0.data(), q_spec, (size_t)n * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    guess_build(t, p0.data(), q0.data());
  }
  if (!G.usable) return false;
  const int Gr = (B + 31) / 32;
  const SchedDev& S = G.dsched.d;
  G.lu.ensure((size_t)Gr * S.n_slots * 32 * 8 + 8);
  G.off.ensure((size_t)Gr * std::max(S.n_off, 1) * 32 * 8);
  G.rhs.ensure((size_t)Gr * G.n2 * 32 * 8);
  G.sol.ensure((size_t)Gr * G.n2 * 32 * 8);
  G.sing.ensure((size_t)Gr * 32 * 4);
  G.piv.ensure((size_t)Gr * 32 * 4);
  G.gact.ensure((size_t)Gr * 4);
  G.err.ensure(16);
  G.gvm.ensure((size_t)B * n * 8);
  G.gva.ensure((size_t)B * n * 8);
  std::vector<int32_t> ones(Gr, 1);
  GOX_CK(cudaMemcpyAsync(G.gact.p, ones.data(), ones.size() * 4, cudaMemcpyHostToDevice, st));
  GOX_CK(cudaMemsetAsync(G.sing.p, 0, (size_t)Gr * 32 * 4, st));
  GOX_CK(cudaMemsetAsync(G.err.p, 0, 16, st));
  const int items = S.n_slots + S.n_off + G.m;
  k_guess_fill<<<dim3((items + 7) / 8, Gr), 256, 0, st>>>(G.d, B, p_spec, q_spec, vm0, va0, v_stride,
                                                          o_slot, o_dre, o_dim, G.lu.as<double>(),
                                                          G.off.as<double>(), G.rhs.as<double>());
  BatchDev D{};
  D.G = Gr;
  D.jbuf = G.lu.p; D.lu = G.lu.p; D.off = G.off.p; D.rhs = G.rhs.p; D.sol = G.sol.p;
  D.sing = G.sing.as<int32_t>(); D.piv_flag = G.piv.as<int32_t>(); D.gact = G.gact.as<int32_t>();
  D.piv_tol = 0.0f;
  D.err = G.err.as<int32_t>();
  Iter<double>::refactor(G.dsched, D, st);
  Iter<double>::solve_rest(G.dsched, D, st);
  k_guess_start<<<grid1d((size_t)B * n), 256, 0, st>>>(B, n, vm0, va0, v_stride, G.gvm.as<double>(),
                                                       G.gva.as<double>());
  k_guess_out<<<grid1d((size_t)B * G.m), 256, 0, st>>>(G.d, B, G.sol.as<double>(), G.sing.as<int32_t>(),
                                                       G.gvm.as<double>(), G.gva.as<double>());
  t->launches += 5;
  int32_t werr = 0;
  GOX_CK(cudaMemcpyAsync(&werr, G.err.p, 4, cudaMemcpyDeviceToHost, st));
  GOX_CK(cudaStreamSynchronize(st));
  GOX_CK(cudaGetLastError());
  if (werr) throw std::runtime_error("a bounded device wait of the guess refactor gave up");
  return true;
}

// When no Jacobian is ever needed (every scenario meets tol at its start),
// or max_iter == 0, the result is computed on the host from the mismatch
// only; no factorization exists to run on the device.
static void host_only_result(gox_topo* t, int B, const double* p_spec, const double* q_spec,
                             const double* vm0, const double* va0, int v_stride,
                             const int32_t* o_slot, const double* o_dre, const double* o_dim,
                             double tol, int max_iter, double* vm_out, double* va_out,
                             int32_t* iters, int32_t* status, double* max_mis, double* hist,
                             const std::vector<int>& singular_first) {
  const int n = t->n_bus;
  std::vector<double> p(n), q(n), yre, yim;
  for (int s = 0; s < B; s++) {
    const double* vm = vm0 + (size_t)s * v_stride;
    const double* va = va0 + (size_t)s * v_stride;
    std::copy(vm, vm + n, vm_out + (size_t)s * n);
    std::copy(va, va + n, va_out + (size_t)s * n);
    if (hist) std::fill(hist + (size_t)s * max_iter, hist + (size_t)(s + 1) * max_iter, 0.0);
    if (max_iter == 0) { iters[s] = 0; status[s] = GOX_MAX_ITERATIONS; max_mis[s] = 0.0; continue; }
    yre = t->yre; yim = t->yim;
    if (o_slot && o_slot[4 * s] >= 0)
      for (int c = 0; c < 4; c++) { yre[o_slot[4 * s + c]] += o_dre[4 * s + c]; yim[o_slot[4 * s + c]] += o_dim[4 * s + c]; }
    host_injections(n, t->yp.data(), t->yi.data(), yre.data(), yim.data(), vm, va, p.data(), q.data());
    double mx = 0.0;
    for (int a = 0; a < t->jac.n_ang; a++) {
      const int i = t->jac.ns_idx[a];
      mx = std::fmax(mx, std::fabs(t->eff(0, i, p_spec[(size_t)s * n + i], vm[i]) - p[i]));
    }
    for (int a = 0; a < t->jac.n_pq; a++) {
      const int i = t->jac.pq_idx[a];
      mx = std::fmax(mx, std::fabs(t->eff(1, i, q_spec[(size_t)s * n + i], vm[i]) - q[i]));
    }
    iters[s] = 1;
    max_mis[s] = mx;
    if (hist) hist[(size_t)s * max_iter] = mx;
    status[s] = mx < tol ? GOX_CONVERGED : GOX_SINGULAR_SCENARIO;
  }
  (void)singular_first;
}


static int batch_device(gox_topo* t, int B, const double* p_spec, const double* q_spec,
                        const double* vm0, const double* va0, int v_stride,
                        const int32_t* o_slot, const double* o_dre, const double* o_dim,
                        double tol, int max_iter, int precision, double* vm_out,
                        double* va_out, int32_t* iters, int32_t* status, double* max_mis,
                        double* hist, cudaStream_t st, const double* h_p, const double* h_q,
                        const double* h_vm, const double* h_va, const int32_t* h_oslot,
                        const double* h_odre, const double* h_odim);

// One batch's device state between its set-up and its results.
struct BatchRun {
  BatchDev D{};
  bool outage = false, want_hist = false;
  bool resolved = false;  // answered without a Newton loop (no Jacobian needed)
};

// The set-up of a batched solve: the linear guess, the pivot order (the
// first solve of a topology), the schedule and streams on the device, the
// batch buffers, the inputs in the interleaved layout, the outages.
static int batch_prepare(gox_topo* t, int B, const double* p_spec, const double* q_spec,
                        const double* vm0, const double* va0, int v_stride,
                        const int32_t* o_slot, const double* o_dre, const double* o_dim,
                        double tol, int max_iter, int precision, double* vm_out,
                        double* va_out, int32_t* iters, int32_t* status, double* max_mis,
                        double* hist, cudaStream_t st, const double* h_p, const double* h_q,
                        const double* h_vm, const double* h_va, const int32_t* h_oslot,
                        const double* h_odre, const double* h_odim, BatchRun& R) {
  const int n = t->n_bus;
  const int G = (B + 31) / 32;
  t->launches = 0;
  const double* zipd = t->zip.empty() ? nullptr : t->dzip.as<double>();
  t->dsched.d.zip = zipd;
  t->guess.d.zip = zipd;
  // the linear initial guess replaces the start points (BatchSolver runs it
  // before every scenario, src/batch.rs:268)
  if (t->guess_mode == 1 &&
      guess_run(t, B, p_spec, q_spec, vm0, va0, v_stride, o_slot, o_dre, o_dim, st)) {
    vm0 = t->guess.gvm.as<double>();
    va0 = t->guess.gva.as<double>();
    v_stride = n;
    h_vm = h_va = nullptr;
    h_p = h_q = nullptr;  // the pivot search reads every input back from the device
    h_oslot = nullptr; h_odre = nullptr; h_odim = nullptr;
  }
  std::vector<int> first_singular;
  if (!t->factored) {
    // host copies of the inputs to find the pivot-fixing Jacobian
    std::vector<double> hp, hq, hvm, hva, hdre, hdim;
    std::vector<int32_t> hslot;
    const double *pp = h_p, *qq = h_q, *vv = h_vm, *aa = h_va, *dr = h_odre, *di = h_odim;
    const int32_t* ss = h_oslot;
    if (!pp) {
      size_t nv = (size_t)(v_stride ? B : 1) * n;
      hp.resize((size_t)B * n); hq.resize((size_t)B * n); hvm.resize(nv); hva.resize(nv);
      GOX_CK(cudaMemcpyAsync(hp.data(), p_spec, hp.size() * 8, cudaMemcpyDeviceToHost, st));
      GOX_CK(cudaMemcpyAsync(hq.data(), q_spec, hq.size() * 8, cudaMemcpyDeviceToHost, st));
      GOX_CK(cudaMemcpyAsync(hvm.data(), vm0, nv * 8, cudaMemcpyDeviceToHost, st));
      GOX_CK(cudaMemcpyAsync(hva.data(), va0, nv * 8, cudaMemcpyDeviceToHost, st));
      if (o_slot) {
        hslot.resize((size_t)B * 4); hdre.resize((size_t)B * 4); hdim.resize((size_t)B * 4);
        GOX_CK(cudaMemcpyAsync(hslot.data(), o_slot, hslot.size() * 4, cudaMemcpyDeviceToHost, st));
        GOX_CK(cudaMemcpyAsync(hdre.data(), o_dre, hdre.size() * 8, cudaMemcpyDeviceToHost, st));
        GOX_CK(cudaMemcpyAsync(hdim.data(), o_dim, hdim.size() * 8, cudaMemcpyDeviceToHost, st));
        ss = hslot.data(); dr = hdre.data(); di = hdim.data();
      }
      GOX_CK(cudaStreamSynchronize(st));
      pp = hp.data(); qq = hq.data(); vv = hvm.data(); aa = hva.data();
    }
    fix_pivots(t, B, pp, qq, vv, aa, v_stride, ss, dr, di, tol, first_singular);
    if (!t->factored) {
      // no Jacobian needed (every scenario meets tol at its start point, e.g.
      // the linear guess of a network without loads) or every candidate
      // factorization was singular: the mismatch at the start points decides
      // Converged or Singular, evaluated on the host copies above (the start
      // points actually used, the guess included)
      std::vector<double> ovm((size_t)B * n), ova((size_t)B * n), mm(B),
          hh(hist ? (size_t)B * max_iter : 0);
      std::vector<int32_t> it(B), stt(B);
      host_only_result(t, B, pp, qq, vv, aa, v_stride, ss, dr, di, tol, max_iter, ovm.data(),
                       ova.data(), it.data(), stt.data(), mm.data(), hist ? hh.data() : nullptr,
                       first_singular);
      GOX_CK(cudaMemcpyAsync(vm_out, ovm.data(), ovm.size() * 8, cudaMemcpyHostToDevice, st));
      GOX_CK(cudaMemcpyAsync(va_out, ova.data(), ova.size() * 8, cudaMemcpyHostToDevice, st));
      GOX_CK(cudaMemcpyAsync(iters, it.data(), (size_t)B * 4, cudaMemcpyHostToDevice, st));
      GOX_CK(cudaMemcpyAsync(status, stt.data(), (size_t)B * 4, cudaMemcpyHostToDevice, st));
      GOX_CK(cudaMemcpyAsync(max_mis, mm.data(), (size_t)B * 8, cudaMemcpyHostToDevice, st));
      if (hist) GOX_CK(cudaMemcpyAsync(hist, hh.data(), hh.size() * 8, cudaMemcpyHostToDevice, st));
      GOX_CK(cudaStreamSynchronize(st));
      R.resolved = true;
      return GOX_OK;
    }
  }
  const bool outage = o_slot != nullptr;
  const bool want_hist = hist != nullptr;
  if (!t->uploaded) {
    t->dsched.load(t->sc, t->yp, t->yi, t->yre, t->yim);
    t->dsched.load_streams(t->s32, t->s64);
    t->uploaded = true;
  }
  const SchedDev& S = t->dsched.d;
  DevBatch& DB = t->batch;
  DB.ensure(S, G, precision, max_iter, want_hist);
  BatchDev D = DB.view(want_hist, outage, tol, t->piv_tol);
  // inputs -> interleaved layout
  const size_t tot = (size_t)G * n * 32;
  k_scatter_rows<<<grid1d(tot), 256, 0, st>>>(p_spec, B, n, n, D.psp, G);
  k_scatter_rows<<<grid1d(tot), 256, 0, st>>>(q_spec, B, n, n, D.qsp, G);
  k_scatter_rows<<<grid1d(tot), 256, 0, st>>>(vm0, B, n, v_stride, D.vm, G);
  k_scatter_rows<<<grid1d(tot), 256, 0, st>>>(va0, B, n, v_stride, D.va, G);
  k_init_scen<<<(G * 32 + 255) / 256, 256, 0, st>>>(B, G, D.status, D.iters, D.sing, D.piv_flag,
                                                     D.maxmis, D.maxacc);
  t->launches += 5;
  if (want_hist) GOX_CK(cudaMemsetAsync(D.hist, 0, (size_t)G * 32 * max_iter * 8, st));
  if (outage) {
    GOX_CK(cudaMemsetAsync(DB.err.p, 0, 4, st));
    k_outage_prep<<<(G * 32 + 255) / 256, 256, 0, st>>>(
        B, G, o_slot, o_dre, o_dim, S.yp, S.yi, n, S.nnz_y, DB.o_slot.as<int32_t>(), DB.o_dre.as<double>(),
        DB.o_dim.as<double>(), DB.o_bf.as<int32_t>(), DB.o_bt.as<int32_t>(), DB.err.as<int32_t>());
    t->launches++;
    int32_t herr = 0;
    GOX_CK(cudaMemcpyAsync(&herr, DB.err.p, 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    if (herr) return GOX_E_BUS_RANGE;
  }
  // scenarios whose own first Jacobian was singular before the pivot order
  // was fixed report Singular after their first mismatch (src/solver.rs:711-716)
  if (!first_singular.empty()) {
    std::vector<int32_t> ones(1, 2);
    for (int s : first_singular)
      GOX_CK(cudaMemcpyAsync(D.sing + s, ones.data(), 4, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaStreamSynchronize(st));
  }
  GOX_CK(cudaMemsetAsync(DB.err.p, 0, 16, st));
  // the running-group count read back every iteration: pinned, kept by the
  // topology (freeing pinned memory synchronizes the whole device, which
  // would stall every other topology's solve in flight)
  if (!t->h_nactive) GOX_CK(cudaMallocHost(&t->h_nactive, sizeof(int32_t)));
  R.D = D;
  R.outage = outage;
  R.want_hist = want_hist;
  return GOX_OK;
}

// The results of a batched solve after its Newton loop: bounded-wait
// errors, outputs in the row-major layout, the mixed path's FP64 re-solves
// of scenarios that tripped the pivot-ratio check.
static int batch_finish(gox_topo* t, int B, const double* p_spec, const double* q_spec,
                        const double* vm0, const double* va0, int v_stride,
                        const int32_t* o_slot, const double* o_dre, const double* o_dim,
                        double tol, int max_iter, int precision, double* vm_out,
                        double* va_out, int32_t* iters, int32_t* status, double* max_mis,
                        double* hist, cudaStream_t st, const double* /*h_p*/,
                        const double* /*h_q*/, const double* /*h_vm*/, const double* /*h_va*/,
                        const int32_t* /*h_oslot*/, const double* /*h_odre*/,
                        const double* /*h_odim*/, BatchRun& R) {
  // (the host copies of the inputs, batch_prepare's, are not read here)
  const int n = t->n_bus;
  const int G = (B + 31) / 32;
  const BatchDev& D = R.D;
  const bool outage = R.outage, want_hist = R.want_hist;
  DevBatch& DB = t->batch;
  {
    int32_t herr[2] = {0, 0};
    GOX_CK(cudaMemcpyAsync(herr, DB.err.p, 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    if (herr[1]) return GOX_E_DEVICE_WAIT;
  }
  // outputs
  k_gather_rows<<<grid1d((size_t)B * n), 256, 0, st>>>(D.vm, B, n, G, vm_out);
  k_gather_rows<<<grid1d((size_t)B * n), 256, 0, st>>>(D.va, B, n, G, va_out);
  k_unpack_scen<<<(B + 255) / 256, 256, 0, st>>>(B, D.status, D.iters, D.maxmis, D.hist,
                                                  max_iter, status, iters, max_mis, hist);
  t->launches += 3;
  GOX_CK(cudaGetLastError());
  if (precision == GOX_PRECISION_MIXED) {
    // Scenarios whose FP32 refactor met a pivot below piv_tol times its
    // column's largest L entry are solved again, from their start point, on
    // the FP64 path (the same pivot order, as the reference's FP64 refactor
    // keeps it); their reports replace the mixed ones.
    std::vector<int32_t> hpiv((size_t)G * 32, 0);
    GOX_CK(cudaMemcpyAsync(hpiv.data(), D.piv_flag, hpiv.size() * 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    std::vector<int32_t> idx;
    for (int s = 0; s < B; s++)
      if (hpiv[s]) idx.push_back(s);
    t->fallbacks = (int64_t)idx.size();
    if (!idx.empty()) {
      const int Bf = (int)idx.size();
      const int64_t launches0 = t->launches;
      const Timing timing0 = t->timing;
      // staging kept by the topology (grow-only): freeing device memory per
      // call would synchronize the whole device under concurrent solves
      FallbackBufs& F = t->fb;
      DevMem &didx = F.idx, &fp = F.p, &fq = F.q, &fvm = F.vm, &fva = F.va, &fsl = F.sl, &fdr = F.dr,
             &fdi = F.di, &ovm = F.ovm, &ova = F.ova, &oit = F.it, &ost = F.st, &omm = F.mm, &ohi = F.hi;
      upload(didx, idx);
      const int32_t* ix = didx.as<int32_t>();
      const size_t rows = (size_t)Bf * n;
      fp.ensure(rows * 8); fq.ensure(rows * 8);
      k_take_rows<double><<<grid1d(rows), 256, 0, st>>>(p_spec, n, ix, Bf, fp.as<double>());
      k_take_rows<double><<<grid1d(rows), 256, 0, st>>>(q_spec, n, ix, Bf, fq.as<double>());
      const double* vmf = vm0;
      const double* vaf = va0;
      if (v_stride) {
        fvm.ensure(rows * 8); fva.ensure(rows * 8);
        k_take_rows<double><<<grid1d(rows), 256, 0, st>>>(vm0, v_stride, ix, Bf, fvm.as<double>());
        k_take_rows<double><<<grid1d(rows), 256, 0, st>>>(va0, v_stride, ix, Bf, fva.as<double>());
        vmf = fvm.as<double>();
        vaf = fva.as<double>();
      }
      if (outage) {
        fsl.ensure((size_t)Bf * 16); fdr.ensure((size_t)Bf * 32); fdi.ensure((size_t)Bf * 32);
        k_take_rows<int32_t><<<grid1d((size_t)Bf * 4), 256, 0, st>>>(o_slot, 4, ix, Bf, fsl.as<int32_t>());
        k_take_rows<double><<<grid1d((size_t)Bf * 4), 256, 0, st>>>(o_dre, 4, ix, Bf, fdr.as<double>());
        k_take_rows<double><<<grid1d((size_t)Bf * 4), 256, 0, st>>>(o_dim, 4, ix, Bf, fdi.as<double>());
      }
      ovm.ensure(rows * 8); ova.ensure(rows * 8);
      oit.ensure((size_t)Bf * 4); ost.ensure((size_t)Bf * 4); omm.ensure((size_t)Bf * 8);
      if (want_hist) ohi.ensure((size_t)Bf * max_iter * 8);
      const int gm = t->guess_mode;
      t->guess_mode = 0;  // the start points are already the guessed ones
      // their static pivot order is poor for their own Jacobians: every
      // Newton step of the re-solve factors with threshold partial pivoting
      struct PivotPass {
        gox_topo* t;
        explicit PivotPass(gox_topo* t_) : t(t_) { t->pivot_pass = true; }
        ~PivotPass() { t->pivot_pass = false; }
      } pivot_scope(t);
      const int rc = batch_device(
          t, Bf, fp.as<double>(), fq.as<double>(), vmf, vaf, v_stride,
          outage ? fsl.as<int32_t>() : nullptr, outage ? fdr.as<double>() : nullptr,
          outage ? fdi.as<double>() : nullptr, tol, max_iter, GOX_PRECISION_FP64, ovm.as<double>(),
          ova.as<double>(), oit.as<int32_t>(), ost.as<int32_t>(), omm.as<double>(),
          want_hist ? ohi.as<double>() : nullptr, st, nullptr, nullptr, nullptr, nullptr, nullptr,
          nullptr, nullptr);
      t->guess_mode = gm;
      if (rc != GOX_OK) return rc;
      k_put_rows<double><<<grid1d(rows), 256, 0, st>>>(ovm.as<double>(), n, ix, Bf, vm_out);
      k_put_rows<double><<<grid1d(rows), 256, 0, st>>>(ova.as<double>(), n, ix, Bf, va_out);
      k_put_rows<int32_t><<<grid1d(Bf), 256, 0, st>>>(oit.as<int32_t>(), 1, ix, Bf, iters);
      k_put_rows<int32_t><<<grid1d(Bf), 256, 0, st>>>(ost.as<int32_t>(), 1, ix, Bf, status);
      k_put_rows<double><<<grid1d(Bf), 256, 0, st>>>(omm.as<double>(), 1, ix, Bf, max_mis);
      if (want_hist)
        k_put_rows<double><<<grid1d((size_t)Bf * max_iter), 256, 0, st>>>(ohi.as<double>(), max_iter,
                                                                          ix, Bf, hist);
      GOX_CK(cudaStreamSynchronize(st));
      GOX_CK(cudaGetLastError());
      t->launches += launches0 + 5 + (v_stride ? 2 : 0) + (outage ? 3 : 0) + (want_hist ? 1 : 0) + 2;
      if (timing0.on) {
        t->timing.total += timing0.total;
        t->timing.k1 += timing0.k1; t->timing.k2 += timing0.k2;
        t->timing.k3 += timing0.k3; t->timing.k4 += timing0.k4;
        t->timing.iters = timing0.iters;
      }
      t->fallbacks = Bf;
    }
  }
  return GOX_OK;
}

static int batch_device(gox_topo* t, int B, const double* p_spec, const double* q_spec,
                        const double* vm0, const double* va0, int v_stride,
                        const int32_t* o_slot, const double* o_dre, const double* o_dim,
                        double tol, int max_iter, int precision, double* vm_out,
                        double* va_out, int32_t* iters, int32_t* status, double* max_mis,
                        double* hist, cudaStream_t st, const double* h_p, const double* h_q,
                        const double* h_vm, const double* h_va, const int32_t* h_oslot,
                        const double* h_odre, const double* h_odim) {
  BatchRun R;
  int rc = batch_prepare(t, B, p_spec, q_spec, vm0, va0, v_stride, o_slot, o_dre, o_dim, tol,
                         max_iter, precision, vm_out, va_out, iters, status, max_mis, hist, st, h_p,
                         h_q, h_vm, h_va, h_oslot, h_odre, h_odim, R);
  if (rc != GOX_OK || R.resolved) return rc;
  if (precision == GOX_PRECISION_FP64)
    run_iterations<double>(t, R.D, max_iter, R.outage, st, t->h_nactive);
  else
    run_iterations<float>(t, R.D, max_iter, R.outage, st, t->h_nactive);
  return batch_finish(t, B, p_spec, q_spec, vm0, va0, v_stride, o_slot, o_dre, o_dim, tol, max_iter,
                      precision, vm_out, va_out, iters, status, max_mis, hist, st, h_p, h_q, h_vm,
                      h_va, h_oslot, h_odre, h_odim, R);
}

// ---------------------------------------------------------------------------
// Many topologies, one Newton loop (the reference's shared work queue over
// uneven scenarios, src/batch.rs:230-281, as one launch per phase).  Every
// topology's batch is set up as for a single solve; then each iteration
// runs the update, injection and decision kernels once over the work items
// {job, block, group} of every topology still running, reads every job's
// running-group count back at once, and runs the fill and the refactor once
// over the running jobs' items (the refactor's CTAs listed largest job
// first, so the longest dependency chains start first; each CTA is sized
// for the largest plan and runs its own job's stream).  A job leaves the
// loop at the iteration its single solve would have left it, with the same
// kernels on the same lanes: its results are the single solve's, bit for
// bit.  The wide kernels' levels run one launch per level over the jobs
// whose plans have that level; only the separate solve of a topology with
// off-diagonal BTF blocks runs per job.
// The lists one iteration's launches run over, for a set of running jobs:
// per kernel the jobs (the refactor's longest first) and the prefix of
// their CTAs; per wide level the jobs whose plans have it.  All lists live
// in one device buffer, rebuilt when a job leaves.
struct MultiLists {
  std::vector<int32_t> host;
  DevMem dev;
  struct L { size_t off = 0, job = 0; int n = 0, ctas = 0; };
  L upd, inj, dec, fill, rf;
  std::vector<L> wide;  // per wide level
  MultiList view(const L& l) const {
    MultiList m;
    m.off = dev.as<int32_t>() + l.off;
    m.job = dev.as<int32_t>() + l.job;
    m.n = l.n;
    return m;
  }
};

template <typename T>
static void build_lists(const std::vector<gox_topo*>& ts, const std::vector<BatchRun>& runs,
                        const std::vector<int>& act, MultiLists& M, cudaStream_t st) {
  const int i = sizeof(T) == 4 ? 0 : 1;
  M.host.clear();
  auto add = [&](const std::vector<int>& jobs, auto ctas_of) {
    MultiLists::L l;
    l.n = (int)jobs.size();
    l.off = M.host.size();
    int c = 0;
    for (int j : jobs) {
      M.host.push_back(c);
      c += ctas_of(j);
    }
    M.host.push_back(c);
    l.job = M.host.size();
    for (int j : jobs) M.host.push_back(j);
    l.ctas = c;
    return l;
  };
  auto G = [&](int j) { return runs[j].D.G; };
  M.upd = add(act, [&](int j) { return update_blocks(ts[j]->dsched.d.n_bus) * G(j); });
  M.inj = add(act, [&](int j) { return inject_blocks(ts[j]->dsched.d.n_bus) * G(j); });
  M.dec = add(act, [&](int j) { return G(j); });
  M.fill = add(act, [&](int j) {
    return fill_blocks(ts[j]->dsched.d.n_ftask, ts[j]->dsched.d.n_fzero) * G(j);
  });
  std::vector<int> order(act);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return (i == 0 ? ts[a]->s32 : ts[a]->s64).est_cycles > (i == 0 ? ts[b]->s32 : ts[b]->s64).est_cycles;
  });
  M.rf = add(order, [&](int j) { return G(j); });
  int maxl = 0;
  for (int j : act) maxl = std::max(maxl, ts[j]->dsched.st_wl[i]);
  M.wide.clear();
  for (int L = 0; L < maxl; L++) {
    std::vector<int> jl;
    for (int j : act)
      if (ts[j]->dsched.st_wl[i] > L) jl.push_back(j);
    M.wide.push_back(add(jl, [&](int j) {
      const std::vector<int32_t>& lp = ts[j]->dsched.lev_ptr_h;
      const long long tasks = (long long)(lp[L + 1] - lp[L]) * G(j);
      return (int)((tasks + kWideWarps - 1) / kWideWarps);
    }));
  }
  M.dev.ensure(M.host.size() * 4);
  GOX_CK(cudaMemcpyAsync(M.dev.p, M.host.data(), M.host.size() * 4, cudaMemcpyHostToDevice, st));
  GOX_CK(cudaStreamSynchronize(st));  // the host vector is rebuilt next time
}

template <typename T>
static void upload_jobs(const std::vector<gox_topo*>& ts, const std::vector<BatchRun>& runs,
                        DevMem& dev, cudaStream_t st) {
  const int i = sizeof(T) == 4 ? 0 : 1;
  std::vector<MultiJob> jobs(ts.size());
  for (size_t j = 0; j < ts.size(); j++) {
    jobs[j].S = ts[j]->dsched.d;
    jobs[j].D = runs[j].D;
    jobs[j].P = ts[j]->dsched.st[i];
    jobs[j].nw = ts[j]->dsched.st_nw[i];
  }
  dev.ensure(jobs.size() * sizeof(MultiJob));
  GOX_CK(cudaMemcpyAsync(dev.p, jobs.data(), jobs.size() * sizeof(MultiJob), cudaMemcpyHostToDevice,
                         st));
  GOX_CK(cudaStreamSynchronize(st));  // the host vector goes out of scope
}

template <typename T>
static void run_multi(const std::vector<gox_topo*>& ts, std::vector<BatchRun>& runs, int max_iter,
                      cudaStream_t st, int64_t& launches) {
  const int nj = (int)ts.size(), i = sizeof(T) == 4 ? 0 : 1;
  DevMem jobs, counts;
  MultiLists M;
  counts.ensure((size_t)nj * 4);
  std::vector<int32_t> h_counts(nj, 0);
  std::vector<int> act(nj);
  for (int j = 0; j < nj; j++) act[j] = j;
  upload_jobs<T>(ts, runs, jobs, st);
  build_lists<T>(ts, runs, act, M, st);
  // the refactor's CTA: the largest plan among the jobs
  int nw_max = 1;
  size_t smem_max = 0;
  auto plan_size = [&]() {
    nw_max = 1;
    smem_max = 0;
    for (gox_topo* t : ts) {
      nw_max = std::max(nw_max, t->dsched.st_nw[i]);
      smem_max = std::max(smem_max, t->dsched.st_smem[i]);
    }
  };
  plan_size();
  {
    static std::once_flag once[64];
    int dev = 0;
    GOX_CK(cudaGetDevice(&dev));
    std::call_once(once[dev & 63], [] {
      GOX_CK(cudaFuncSetAttribute(k_refactor_multi<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kRefactorSmem));
      GOX_CK(cudaFuncSetAttribute(k_refactor_wide_multi<T>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)Iter<T>::kWideSmem));
    });
  }
  const MultiJob* J = nullptr;
  auto count = [&](int zero) {
    k_multi_counts<<<(nj + 127) / 128, 128, 0, st>>>(jobs.as<MultiJob>(), nj, counts.as<int32_t>(),
                                                       zero);
    launches++;
  };
  auto launch = [&](const MultiLists::L& l, auto kernel_launch) {
    if (l.n > 0 && l.ctas > 0) {
      kernel_launch((unsigned)l.ctas, M.view(l));
      launches++;
    }
  };
  // CUDA events around the phases when the first topology's timing is on:
  // its report holds the loop's mismatch (k1), fill (k2), shared refactor
  // launch (k3) and wide levels around it (k4)
  const bool timing = ts[0]->timing.on;
  std::vector<cudaEvent_t> ev;
  auto rec = [&]() {
    if (!timing) return;
    cudaEvent_t e;
    GOX_CK(cudaEventCreate(&e));
    GOX_CK(cudaEventRecord(e, st));
    ev.push_back(e);
  };
  int it = 0;
  for (it = 0; it < max_iter && !act.empty(); it++) {
    J = jobs.as<MultiJob>();
    rec();
    count(1);
    launch(M.upd, [&](unsigned c, MultiList l) { k_update_multi<T><<<c, 256, 0, st>>>(J, l, it, 0); });
    launch(M.inj, [&](unsigned c, MultiList l) { k_inject_multi<T><<<c, 256, 0, st>>>(J, l, it); });
    launch(M.dec, [&](unsigned c, MultiList l) { k_decide_multi<<<c, 32, 0, st>>>(J, l, it, 0); });
    count(0);
    rec();
    GOX_CK(cudaMemcpyAsync(h_counts.data(), counts.p, (size_t)nj * 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    std::vector<int> still;
    for (int j : act)
      if (h_counts[j] > 0) still.push_back(j);
    if (still.size() != act.size()) {
      act.swap(still);
      if (act.empty()) break;
      build_lists<T>(ts, runs, act, M, st);
    }
    rec();
    launch(M.fill, [&](unsigned c, MultiList l) { k_fill_multi<T><<<c, 32 * kWarps, 0, st>>>(J, l); });
    rec();
    // a job whose plan was not timed yet: the autotuner, as its single
    // solve would run it here
    bool retuned = false;
    for (int j : act)
      if (!ts[j]->tune[i].done) {
        autotune<T>(ts[j], runs[j].D, st);
        retuned = true;
      }
    if (retuned) {
      upload_jobs<T>(ts, runs, jobs, st);
      build_lists<T>(ts, runs, act, M, st);
      plan_size();
      J = jobs.as<MultiJob>();
    }
    rec();
    int wr = 1;
    for (int j : act) wr = std::max(wr, ts[j]->dsched.st_wr[i]);
    for (size_t L = 0; L < M.wide.size(); L++)
      launch(M.wide[L], [&](unsigned c, MultiList l) {
        k_refactor_wide_multi<T><<<c, 32 * kWideWarps, Iter<T>::wide_smem(wr), st>>>(J, l, (int)L, wr);
      });
    rec();
    launch(M.rf, [&](unsigned c, MultiList l) {
      k_refactor_multi<T><<<c, 32 * nw_max, smem_max, st>>>(J, l);
    });
    rec();
    for (size_t L = M.wide.size(); L-- > 0;)
      launch(M.wide[L], [&](unsigned c, MultiList l) {
        k_solve_wide_multi<T><<<c, 32 * kWideWarps, 0, st>>>(J, l, (int)L);
      });
    for (int j : act) launches += Iter<T>::solve_rest(ts[j]->dsched, runs[j].D, st);
    rec();
    GOX_CK(cudaGetLastError());
  }
  if (it == max_iter && !act.empty()) {
    // the budget ran out with scenarios still running: their MaxIterations
    // mismatch (update and decision, as the single solve's last step)
    J = jobs.as<MultiJob>();
    launch(M.upd, [&](unsigned c, MultiList l) {
      k_update_multi<T><<<c, 256, 0, st>>>(J, l, max_iter, 1);
    });
    launch(M.dec, [&](unsigned c, MultiList l) {
      k_decide_multi<<<c, 32, 0, st>>>(J, l, max_iter, 1);
    });
  }
  GOX_CK(cudaStreamSynchronize(st));
  GOX_CK(cudaGetLastError());
  if (timing && ev.size() >= 2) {
    // per full iteration 8 events: [0] mismatch [1] | [2] fill [3] | [4]
    // wide levels [5] refactor [6] wide backward levels [7]; the last
    // iteration may stop after [1]
    auto el = [&](size_t a, size_t b) {
      float ms = 0;
      GOX_CK(cudaEventElapsedTime(&ms, ev[a], ev[b]));
      return (double)ms;
    };
    Timing& T_ = ts[0]->timing;
    T_.iters = it;
    T_.total = el(0, ev.size() - 1);
    T_.k1 = T_.k2 = T_.k3 = T_.k4 = 0;
    for (size_t b = 0; b + 1 < ev.size(); b += 8) {
      T_.k1 += el(b, b + 1);
      if (b + 7 >= ev.size()) break;
      T_.k2 += el(b + 2, b + 3);
      T_.k3 += el(b + 5, b + 6);
      T_.k4 += el(b + 4, b + 5) + el(b + 6, b + 7);
    }
    for (auto e : ev) cudaEventDestroy(e);
  }
}

// The persistent form (k_newton_persistent): each group's whole Newton loop
// in one CTA taking (topology, group) items from a queue, largest topology
// first, in one launch for the whole call.  Each topology runs a plan
// without the wide split (FP32 up to 12 warps, FP64 8), compiled and checked
// once.  gox_set_multi_persistent(1) chooses it over the lockstep loop above
// (the default, faster on the many-topology workload: its big grids keep
// their wide kernels, while a persistent CTA runs a big grid's group alone on
// its SM); a topology for which no such plan fits sends the call to the
// lockstep loop.
static std::atomic<int> g_multi_persistent{0};
// dynamic shared memory a persistent plan may use (the kernel's static
// shared memory -- the job, the injections' reduction row, the refactor's
// barriers and flags -- takes the rest of the 227 KB)
static constexpr size_t kPersistSmem = 223 * 1024;

// The persistent kernel's plan of a topology in precision i (built once);
// false when none fits.
static bool persist_plan(gox_topo* t, int i) {
  gox_topo::PersistPlan& PP = t->persist[i];
  if (PP.built) return PP.nw > 0;
  PP.built = true;
  const int elem = i == 0 ? 4 : 8;
  bool ok = false;
  for (const StreamPlan& p : candidate_plans(t->sc, elem, kPersistSmem)) {
    if (p.sync != 0 || p.wide_levels != 0) continue;
    if (compile_checked(t->sc, p, PP.s) && PP.s.has_bwd) {
      ok = true;
      break;
    }
  }
  if (!ok) {
    PP.nw = 0;
    return false;
  }
  upload(PP.words, PP.s.words);
  upload(PP.c0, PP.s.chunk0);
  upload(PP.nc, PP.s.nchunks);
  PP.d = StreamDev{};
  PP.d.words = PP.words.as<int32_t>();
  PP.d.chunk0 = PP.c0.as<int32_t>();
  PP.d.nchunks = PP.nc.as<int32_t>();
  PP.d.ring_rows = PP.s.plan.ring_rows;
  PP.d.rows_total = ring_total(PP.s.plan);
  PP.d.chunk_words = PP.s.plan.chunk_words;
  PP.d.n_bars = PP.s.n_bars;
  PP.d.sync = PP.s.plan.sync;
  PP.nw = PP.s.plan.nw;
  PP.smem = stream_smem_bytes(PP.s.plan);
  return true;
}

template <typename T>
static void run_persistent(const std::vector<gox_topo*>& ts, std::vector<BatchRun>& runs,
                           int max_iter, cudaStream_t st, int64_t& launches) {
  const int nj = (int)ts.size(), i = sizeof(T) == 4 ? 0 : 1;
  std::vector<MultiJob> jobs(nj);
  size_t smem = 0;
  int nw = 8;
  for (int j = 0; j < nj; j++) {
    jobs[j].S = ts[j]->dsched.d;
    jobs[j].D = runs[j].D;
    jobs[j].P = ts[j]->persist[i].d;
    jobs[j].nw = ts[j]->persist[i].nw;
    smem = std::max(smem, ts[j]->persist[i].smem);
    nw = std::max(nw, ts[j]->persist[i].nw);
  }
  // items: every group of every job, the longest jobs first
  std::vector<int> order(nj);
  for (int j = 0; j < nj; j++) order[j] = j;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return ts[a]->persist[i].s.est_cycles > ts[b]->persist[i].s.est_cycles;
  });
  std::vector<int2> items;
  for (int j : order)
    for (int g = 0; g < runs[j].D.G; g++) items.push_back(make_int2(j, g));
  DevMem djobs, ditems, dnext;
  djobs.ensure(jobs.size() * sizeof(MultiJob));
  ditems.ensure(items.size() * sizeof(int2));
  dnext.ensure(sizeof(int));
  GOX_CK(cudaMemcpyAsync(djobs.p, jobs.data(), jobs.size() * sizeof(MultiJob), cudaMemcpyHostToDevice,
                         st));
  GOX_CK(cudaMemcpyAsync(ditems.p, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice,
                         st));
  GOX_CK(cudaMemsetAsync(dnext.p, 0, sizeof(int), st));
  int dev = 0, sms = 0;
  GOX_CK(cudaGetDevice(&dev));
  GOX_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  {
    static std::once_flag once[64];
    std::call_once(once[dev & 63], [] {
      GOX_CK(cudaFuncSetAttribute(k_newton_persistent<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kPersistSmem));
    });
  }
  const int grid = (int)std::min<size_t>(items.size(), (size_t)sms);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const bool timing = ts[0]->timing.on;
  if (timing) {
    GOX_CK(cudaEventCreate(&e0));
    GOX_CK(cudaEventCreate(&e1));
    GOX_CK(cudaEventRecord(e0, st));
  }
  k_newton_persistent<T><<<grid, 32 * nw, smem, st>>>(
      djobs.as<MultiJob>(), ditems.as<int2>(), (int)items.size(), dnext.as<int>(), max_iter);
  launches++;
  if (timing) GOX_CK(cudaEventRecord(e1, st));
  GOX_CK(cudaStreamSynchronize(st));  // the host vectors go out of scope
  GOX_CK(cudaGetLastError());
  if (timing) {
    float ms = 0;
    GOX_CK(cudaEventElapsedTime(&ms, e0, e1));
    Timing& T_ = ts[0]->timing;
    T_.total = ms;
    T_.k1 = T_.k2 = T_.k4 = 0;
    T_.k3 = ms;  // one launch: every phase of every group
    T_.iters = 0;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
}

// ---------------------------------------------------------------------------
// Q-limit enforcement (newton_raphson_enforcing_q_limits, src/solver.rs:545-618)
// over a batch: scenarios are grouped by the set of PV buses they have
// switched to PQ, each group solved on the topology variant with those bus
// types, warm started from its previous state.

// Computed Q of buses `bus[k]` for every scenario, from row-major V [B][N]
__global__ void k_qcalc(int B, int N, const int32_t* __restrict__ yp, const int32_t* __restrict__ yi,
                        const double* __restrict__ yre, const double* __restrict__ yim,
                        const double* __restrict__ vm, const double* __restrict__ va,
                        const int32_t* __restrict__ bus, int nb, double* __restrict__ qout) {
  const size_t total = (size_t)B * nb;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int s = (int)(t / nb), i = bus[t % nb];
    const double* vms = vm + (size_t)s * N;
    const double* vas = va + (size_t)s * N;
    double ir = 0.0, ii = 0.0;
    for (int p = yp[i]; p < yp[i + 1]; p++) {
      const int j = yi[p];
      double sn, cs;
      sincos(vas[j], &sn, &cs);
      const double e = vms[j] * cs, f = vms[j] * sn;
      ir += yre[p] * e - yim[p] * f;
      ii += yre[p] * f + yim[p] * e;
    }
    double sn, cs;
    sincos(vas[i], &sn, &cs);
    const double e = vms[i] * cs, f = vms[i] * sn;
    qout[t] = f * ir - e * ii;
  }
}

// q[s][bus] = value for each pinned (scenario, bus, value)
__global__ void k_pin(int m, const int32_t* __restrict__ sb, const double* __restrict__ val, int N,
                      double* __restrict__ q) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m) q[(size_t)sb[2 * k] * N + sb[2 * k + 1]] = val[k];
}

static constexpr int kQlimWorkers = 8;  // host threads solving switched-set groups

// The variant of `t` whose buses `changes` (sorted, each bus * 4 + its new
// type) have other types: PV buses switched to PQ by their reactive limits,
// the buses of a sourceless island pinned as slack buses.  Built on first use
// (analysis of its own Jacobian) and kept by `t`.
static gox_topo* topo_variant(gox_topo* t, const std::vector<int32_t>& changes) {
  if (changes.empty()) return t;
  for (auto& v : t->variants)
    if (v.first == changes) return v.second;
  std::unique_ptr<gox_topo> v(new gox_topo());
  v->n_bus = t->n_bus;
  v->yp = t->yp; v->yi = t->yi; v->yre = t->yre; v->yim = t->yim;
  v->bus_type = t->bus_type;
  for (int c : changes) v->bus_type[c >> 2] = c & 3;
  v->jac = jac_analyze(v->n_bus, v->yp.data(), v->yi.data(), v->bus_type.data());
  v->csc = build_csc(v->jac.n_u, v->jac.nnz(), v->jac.rows.data(), v->jac.cols.data());
  v->sym = klu_analyze(v->jac.n_u, v->csc.p.data(), v->csc.i.data());
  v->device = t->device;
  v->piv_tol = t->piv_tol;
  v->zip = t->zip;
  if (!v->zip.empty()) upload(v->dzip, v->zip);
  v->tune_cache_only = true;  // many variants solve concurrently: no timing of their own
  t->variants.emplace_back(changes, v.get());
  return v.release();
}

// ---------------------------------------------------------------------------
// Islands of outage scenarios (network::connected_components / classify /
// mark_unreferenced_islands, src/network.rs:121-223): an outage whose
// off-diagonal Y entries become exactly zero removes its edge from the
// graph; when that edge is a bridge the grid splits, and every component
// without a slack bus is pinned to V = 0 (slack type, no injection) for
// that scenario.

// Bridges of the Y-bus graph (iterative Tarjan), as sorted (min, max) pairs
static void find_bridges(gox_topo* t) {
  const int n = t->n_bus;
  std::vector<int32_t> disc(n, -1), low(n, 0), parent_edge(n, -1);
  std::vector<std::pair<int, int>> stack;  // (bus, next entry position)
  int timer = 0;
  t->bridges.clear();
  for (int r = 0; r < n; r++) {
    if (disc[r] >= 0) continue;
    disc[r] = low[r] = timer++;
    stack.push_back({r, t->yp[r]});
    while (!stack.empty()) {
      const int u = stack.back().first;
      int& pos = stack.back().second;
      if (pos < t->yp[u + 1]) {
        const int e = pos++;
        const int w = t->yi[e];
        if (w == u) continue;
        if (disc[w] < 0) {
          parent_edge[w] = u;
          disc[w] = low[w] = timer++;
          stack.push_back({w, t->yp[w]});
        } else if (w != parent_edge[u]) {
          low[u] = std::min(low[u], disc[w]);
        }
      } else {
        stack.pop_back();
        const int pu = parent_edge[u];
        if (pu >= 0) {
          low[pu] = std::min(low[pu], low[u]);
          if (low[u] > disc[pu]) t->bridges.push_back({std::min(pu, u), std::max(pu, u)});
        }
      }
    }
  }
  std::sort(t->bridges.begin(), t->bridges.end());
  t->bridges_found = true;
}

// Components (connected_components order: by smallest member) of the graph
// without edge (a, b): label per bus
static std::vector<int32_t> components_without(const gox_topo* t, int a, int b) {
  const int n = t->n_bus;
  std::vector<int32_t> label(n, -1), stack;
  int nc = 0;
  for (int r = 0; r < n; r++) {
    if (label[r] >= 0) continue;
    label[r] = nc;
    stack.push_back(r);
    while (!stack.empty()) {
      const int u = stack.back();
      stack.pop_back();
      for (int e = t->yp[u]; e < t->yp[u + 1]; e++) {
        const int w = t->yi[e];
        if (label[w] >= 0 || (u == a && w == b) || (u == b && w == a)) continue;
        label[w] = nc;
        stack.push_back(w);
      }
    }
    nc++;
  }
  return label;
}

// The pinned buses (sorted) of one outage scenario, and its components
// (labels, or empty when the outage does not split the grid)
static const std::vector<int32_t>& outage_split(gox_topo* t, const int32_t* slot, const double* dre,
                                               const double* dim, std::vector<int32_t>* pinned) {
  static const std::vector<int32_t> none;
  pinned->clear();
  if (slot[0] < 0) return none;
  const int nnz = (int)t->yi.size();
  for (int c = 0; c < 4; c++)
    if (slot[c] < 0 || slot[c] >= nnz) throw std::runtime_error("bad outage slot");
  // slots: ff, ft, tf, tt; the edge is gone when both off-diagonals vanish
  if (t->yre[slot[1]] + dre[1] != 0.0 || t->yim[slot[1]] + dim[1] != 0.0 ||
      t->yre[slot[2]] + dre[2] != 0.0 || t->yim[slot[2]] + dim[2] != 0.0)
    return none;
  const int b = t->yi[slot[1]];
  const int a = (int)(std::upper_bound(t->yp.begin(), t->yp.end(), slot[1]) - t->yp.begin()) - 1;
  if (!t->bridges_found) find_bridges(t);
  const std::pair<int, int> key{std::min(a, b), std::max(a, b)};
  if (!std::binary_search(t->bridges.begin(), t->bridges.end(), key)) return none;
  auto it = t->splits.find(key);
  if (it == t->splits.end()) it = t->splits.emplace(key, components_without(t, a, b)).first;
  const std::vector<int32_t>& label = it->second;
  const int nc = 1 + *std::max_element(label.begin(), label.end());
  std::vector<int32_t> slacks(nc, 0);
  for (int i = 0; i < t->n_bus; i++)
    if (t->bus_type[i] == 3) slacks[label[i]]++;
  for (int i = 0; i < t->n_bus; i++)
    if (slacks[label[i]] == 0) pinned->push_back(i);
  return label;
}

// q[s][bus] = 0, p likewise, and V = 0 for the pinned buses of every row
__global__ void k_pin_island(int Bg, int N, const int32_t* __restrict__ bus, int nb, double* p,
                             double* q, double* vm, double* va) {
  const size_t total = (size_t)Bg * nb;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t x = (t / nb) * N + bus[t % nb];
    p[x] = 0.0;
    q[x] = 0.0;
    vm[x] = 0.0;
    va[x] = 0.0;
  }
}

// batch_device with the islands of outage scenarios: scenarios are grouped
// by the buses their outage leaves without a slack bus; a group with pinned
// buses runs on the variant of `t` where they are slack buses at V = 0 with
// no injection (its start rule is t's).  Without splitting outages this is
// batch_device itself.
static int batch_any(gox_topo* t, int B, const double* p_spec, const double* q_spec,
                     const double* vm0, const double* va0, int v_stride, const int32_t* o_slot,
                     const double* o_dre, const double* o_dim, double tol, int max_iter,
                     int precision, double* vm_out, double* va_out, int32_t* iters,
                     int32_t* status, double* max_mis, double* hist, cudaStream_t st,
                     const double* h_p, const double* h_q, const double* h_vm, const double* h_va,
                     const int32_t* h_oslot, const double* h_odre, const double* h_odim) {
  auto whole = [&]() {
    return batch_device(t, B, p_spec, q_spec, vm0, va0, v_stride, o_slot, o_dre, o_dim, tol,
                        max_iter, precision, vm_out, va_out, iters, status, max_mis, hist, st, h_p,
                        h_q, h_vm, h_va, h_oslot, h_odre, h_odim);
  };
  if (!o_slot) return whole();
  std::vector<int32_t> hs;
  std::vector<double> hr, hi;
  const int32_t* ss = h_oslot;
  const double *dr = h_odre, *di = h_odim;
  if (!ss) {
    hs.resize((size_t)B * 4); hr.resize(hs.size()); hi.resize(hs.size());
    GOX_CK(cudaMemcpyAsync(hs.data(), o_slot, hs.size() * 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(hr.data(), o_dre, hr.size() * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(hi.data(), o_dim, hi.size() * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    ss = hs.data(); dr = hr.data(); di = hi.data();
  }
  std::map<std::vector<int32_t>, std::vector<int32_t>> groups;  // pinned buses -> scenarios
  std::vector<int32_t> pinned;
  for (int s = 0; s < B; s++) {
    outage_split(t, ss + 4 * s, dr + 4 * s, di + 4 * s, &pinned);
    groups[pinned].push_back(s);
  }
  if (groups.size() == 1 && groups.begin()->first.empty()) return whole();
  const int n = t->n_bus;
  int64_t launches = 0;
  DevMem dix, dzero, dpin, sp, sq, svm, sva, ssl, sdr, sdi, ovm, ova, oit, ost, omm, ohi;
  for (auto& gk : groups) {
    const std::vector<int32_t>& idx = gk.second;
    const int Bg = (int)idx.size();
    const size_t rows = (size_t)Bg * n;
    upload(dix, idx);
    const int32_t* ix = dix.as<int32_t>();
    sp.ensure(rows * 8); sq.ensure(rows * 8); svm.ensure(rows * 8); sva.ensure(rows * 8);
    ssl.ensure((size_t)Bg * 16); sdr.ensure((size_t)Bg * 32); sdi.ensure((size_t)Bg * 32);
    ovm.ensure(rows * 8); ova.ensure(rows * 8);
    oit.ensure((size_t)Bg * 4); ost.ensure((size_t)Bg * 4); omm.ensure((size_t)Bg * 8);
    if (hist) ohi.ensure((size_t)Bg * max_iter * 8);
    k_take_rows<double><<<grid1d(rows), 256, 0, st>>>(p_spec, n, ix, Bg, sp.as<double>());
    k_take_rows<double><<<grid1d(rows), 256, 0, st>>>(q_spec, n, ix, Bg, sq.as<double>());
    const int32_t* vix = ix;
    if (!v_stride) {  // one shared start row
      upload(dzero, std::vector<int32_t>(Bg, 0));
      vix = dzero.as<int32_t>();
    }
    k_take_rows<double><<<grid1d(rows), 256, 0, st>>>(vm0, n, vix, Bg, svm.as<double>());
    k_take_rows<double><<<grid1d(rows), 256, 0, st>>>(va0, n, vix, Bg, sva.as<double>());
    k_take_rows<int32_t><<<grid1d((size_t)Bg * 4), 256, 0, st>>>(o_slot, 4, ix, Bg, ssl.as<int32_t>());
    k_take_rows<double><<<grid1d((size_t)Bg * 4), 256, 0, st>>>(o_dre, 4, ix, Bg, sdr.as<double>());
    k_take_rows<double><<<grid1d((size_t)Bg * 4), 256, 0, st>>>(o_dim, 4, ix, Bg, sdi.as<double>());
    gox_topo* v = t;
    if (!gk.first.empty()) {
      std::vector<int32_t> changes(gk.first.size());
      for (size_t c = 0; c < changes.size(); c++) changes[c] = gk.first[c] * 4 + 3;  // -> slack
      v = topo_variant(t, changes);
      v->guess_mode = t->guess_mode;
      upload(dpin, gk.first);
      k_pin_island<<<grid1d((size_t)Bg * gk.first.size()), 256, 0, st>>>(
          Bg, n, dpin.as<int32_t>(), (int)gk.first.size(), sp.as<double>(), sq.as<double>(),
          svm.as<double>(), sva.as<double>());
    }
    GOX_CK(cudaGetLastError());
    const int r = batch_device(v, Bg, sp.as<double>(), sq.as<double>(), svm.as<double>(),
                               sva.as<double>(), n, ssl.as<int32_t>(), sdr.as<double>(),
                               sdi.as<double>(), tol, max_iter, precision, ovm.as<double>(),
                               ova.as<double>(), oit.as<int32_t>(), ost.as<int32_t>(),
                               omm.as<double>(), hist ? ohi.as<double>() : nullptr, st, nullptr,
                               nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    if (r != GOX_OK) return r;
    launches += v->launches + 13;
    k_put_rows<double><<<grid1d(rows), 256, 0, st>>>(ovm.as<double>(), n, ix, Bg, vm_out);
    k_put_rows<double><<<grid1d(rows), 256, 0, st>>>(ova.as<double>(), n, ix, Bg, va_out);
    k_put_rows<int32_t><<<grid1d(Bg), 256, 0, st>>>(oit.as<int32_t>(), 1, ix, Bg, iters);
    k_put_rows<int32_t><<<grid1d(Bg), 256, 0, st>>>(ost.as<int32_t>(), 1, ix, Bg, status);
    k_put_rows<double><<<grid1d(Bg), 256, 0, st>>>(omm.as<double>(), 1, ix, Bg, max_mis);
    if (hist)
      k_put_rows<double><<<grid1d((size_t)Bg * max_iter), 256, 0, st>>>(ohi.as<double>(), max_iter, ix,
                                                                        Bg, hist);
    GOX_CK(cudaGetLastError());
    GOX_CK(cudaStreamSynchronize(st));  // the staging buffers are reused by the next group
  }
  t->launches = launches;
  return GOX_OK;
}

// A second instance of a factored topology: the same pattern, pivot order,
// schedule, plans and settings; its own device state (it runs the streams its
// topology chose, so its results are its topology's bit for bit)
static std::unique_ptr<gox_topo> clone_factored(const gox_topo* t) {
  std::unique_ptr<gox_topo> v(new gox_topo());
  v->n_bus = t->n_bus;
  v->yp = t->yp; v->yi = t->yi; v->yre = t->yre; v->yim = t->yim; v->bus_type = t->bus_type;
  v->jac = t->jac; v->csc = t->csc; v->sym = t->sym; v->num = t->num; v->sc = t->sc;
  v->s32 = t->s32; v->s64 = t->s64;
  v->factored = true;
  v->uploaded = false;
  v->device = t->device;
  v->piv_tol = t->piv_tol;
  v->graphs_wanted = t->graphs_wanted;
  v->zip = t->zip;
  if (!v->zip.empty()) upload(v->dzip, v->zip);
  v->tune[0].done = v->tune[1].done = true;
  return v;
}

// The twin a split solve's next part runs on (install_stream keeps its
// streams the topology's)
static gox_topo* split_twin(gox_topo* t) {
  if (!t->twin) t->twin = clone_factored(t);
  return t->twin.get();
}

static constexpr int kSplitMinScenarios = 4096;

// Holds a stream for `ns` nanoseconds (global timer; ns is capped by the
// caller): part k of a split solve starts k offsets later, so that its
// mismatch and fill fall on the other parts' refactors instead of running
// beside their own mismatch.
__global__ void k_delay(unsigned long long ns) {
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  do {
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  } while (t - t0 < ns);
}

// The offset: about two thirds of one part's mismatch and fill, estimated per
// bus and scenario (measured on the 2,000-bus grid: 0.29 ms for parts of
// 2,048 scenarios), at most 5 ms
static unsigned long long split_offset_ns(int n_bus, int scenarios) {
  const double ns = 0.07 * (double)n_bus * (double)scenarios;
  return (unsigned long long)std::min(ns, 5.0e6);
}

// batch_any, or -- when the topology is set to split, its pivot order is
// fixed, the start is given and the batch is large -- its parts (split at
// multiples of 32 scenarios, so every group and result is the same) solved
// concurrently, the first on `st` and each other one by a twin on its own
// stream from its own host thread
static int batch_split(gox_topo* t, int B, const double* p_spec, const double* q_spec,
                       const double* vm0, const double* va0, int v_stride, const int32_t* o_slot,
                       const double* o_dre, const double* o_dim, double tol, int max_iter,
                       int precision, double* vm_out, double* va_out, int32_t* iters,
                       int32_t* status, double* max_mis, double* hist, cudaStream_t st,
                       const double* h_p, const double* h_q, const double* h_vm, const double* h_va,
                       const int32_t* h_oslot, const double* h_odre, const double* h_odim) {
  // (FP64 solves stay whole: their refactor is bound by the FP64 pipe, which
  // the parts would share; measured slower split)
  // (and not before the topology's plan for this precision is tuned: the
  // tuning installs streams the twin shares)
  // by batch size: two parts, four from 8,192 scenarios (measured on the
  // 10,000-bus N-1 batch of 8,192: 4 parts 117-121 ms, 2 parts 122-124 ms
  // with host buffers; the 2,000-bus batch of 4,096 alike for 2, 4 and 8)
  const int want = t->split_parts > 0 ? t->split_parts : (B >= 8192 ? 4 : 2);
  if (want < 2 || !t->factored || t->guess_mode != 0 || t->timing.on ||
      B < kSplitMinScenarios || precision != GOX_PRECISION_MIXED || !t->tune[0].done)
    return batch_any(t, B, p_spec, q_spec, vm0, va0, v_stride, o_slot, o_dre, o_dim, tol, max_iter,
                     precision, vm_out, va_out, iters, status, max_mis, hist, st, h_p, h_q, h_vm,
                     h_va, h_oslot, h_odre, h_odim);
  // parts of whole groups (every group and result is the one the whole
  // batch would have), part k solved by the k-th twin on its own stream from
  // its own host thread, started k offsets later
  const int n = t->n_bus;
  const int parts = std::min(want, (B + 31) / 32);
  const int G = (B + 31) / 32;
  std::vector<int> first(parts + 1, 0);
  for (int k = 0; k < parts; k++) first[k + 1] = first[k] + (G / parts + (k < G % parts ? 1 : 0)) * 32;
  first[parts] = B;
  std::vector<gox_topo*> tw(parts, t);
  for (int k = 1; k < parts; k++) {
    tw[k] = split_twin(tw[k - 1]);
    if (!tw[k]->own_stream) GOX_CK(cudaStreamCreateWithFlags(&tw[k]->own_stream, cudaStreamNonBlocking));
  }
  cudaEvent_t ready;
  GOX_CK(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  GOX_CK(cudaEventRecord(ready, st));  // the inputs, as the caller's stream has them
  std::vector<int> rk(parts, GOX_OK);
  auto part = [&](int k, cudaStream_t sk) -> int {
    const int Bk = first[k + 1] - first[k];
    const size_t off = (size_t)first[k] * n, voff = v_stride ? off : 0;
    const size_t o4 = 4 * (size_t)first[k];
    return batch_any(tw[k], Bk, p_spec + off, q_spec + off, vm0 + voff, va0 + voff, v_stride,
                     o_slot ? o_slot + o4 : nullptr, o_dre ? o_dre + o4 : nullptr,
                     o_dim ? o_dim + o4 : nullptr, tol, max_iter, precision, vm_out + off,
                     va_out + off, iters + first[k], status + first[k], max_mis + first[k],
                     hist ? hist + (size_t)first[k] * max_iter : nullptr, sk,
                     h_p ? h_p + off : nullptr, h_q ? h_q + off : nullptr,
                     h_vm ? h_vm + voff : nullptr, h_va ? h_va + voff : nullptr,
                     h_oslot ? h_oslot + o4 : nullptr, h_odre ? h_odre + o4 : nullptr,
                     h_odim ? h_odim + o4 : nullptr);
  };
  std::vector<std::thread> th;
  for (int k = 1; k < parts; k++)
    th.emplace_back([&, k] {
      rk[k] = guard_impl([&]() -> int {
        GOX_CK(cudaSetDevice(t->device));
        cudaStream_t sk = tw[k]->own_stream;
        AllocStreamScope scope(sk);
        GOX_CK(cudaStreamWaitEvent(sk, ready, 0));
        k_delay<<<1, 1, 0, sk>>>((unsigned long long)k *
                                 split_offset_ns(n, first[k + 1] - first[k]));
        GOX_CK(cudaGetLastError());
        return part(k, sk);
      });
    });
  try {
    rk[0] = part(0, st);
  } catch (...) {
    for (auto& x : th) x.join();
    cudaEventDestroy(ready);
    throw;
  }
  for (auto& x : th) x.join();
  cudaEventDestroy(ready);
  for (int k = 1; k < parts; k++) {
    t->launches += tw[k]->launches + 1;
    t->fallbacks += tw[k]->fallbacks;
  }
  for (int r : rk)
    if (r != GOX_OK) return r;
  return GOX_OK;
}

extern "C" {

const char* gox_version(void) { return "gridoxide_gb300 0.1.0 (sm_103a)"; }

int gox_analyze(int32_t n, const int32_t* Ap, const int32_t* Ai, int32_t* P, int32_t* Q,
                int32_t* R) {
  if (n < 0 || !Ap || !Ai || !P || !Q || !R) return GOX_E_INVALID;
  return guard_impl([&]() -> int {
    for (int j = 0; j < n; j++)
      if (Ap[j] > Ap[j + 1]) return GOX_E_INVALID;
    for (int p = 0; p < Ap[n]; p++)
      if (Ai[p] < 0 || Ai[p] >= n) return GOX_E_INVALID;
    Symbolic S = klu_analyze(n, Ap, Ai);
    std::copy(S.P.begin(), S.P.end(), P);
    std::copy(S.Q.begin(), S.Q.end(), Q);
    std::copy(S.R.begin(), S.R.end(), R);
    return S.nblocks;
  });
}

int gox_factor_host(int32_t n, int32_t nnz, const int32_t* rows, const int32_t* cols,
                    const double* vals, int64_t* sizes, int32_t* Lp, int32_t* Li, double* Lx,
                    int32_t* Up, int32_t* Ui, double* Ux, int32_t* Fp, int32_t* Fi, double* Fx,
                    int32_t* P, int32_t* Q, int32_t* R) {
  if (n <= 0 || nnz < 0 || !sizes || (nnz > 0 && (!rows || !cols || !vals))) return GOX_E_INVALID;
  for (int e = 0; e < nnz; e++)
    if (rows[e] < 0 || rows[e] >= n || cols[e] < 0 || cols[e] >= n) return GOX_E_INVALID;
  return guard_impl([&]() -> int {
    Csc A = build_csc(n, nnz, rows, cols);
    Symbolic S = klu_analyze(n, A.p.data(), A.i.data());
    std::vector<double> packed(A.nnz(), 0.0);
    for (int e = 0; e < nnz; e++) packed[A.slot_of[e]] += vals[e];
    Numeric N;
    if (klu_factor(A, packed.data(), S, 0.001, N) != 0) return GOX_SINGULAR;
    sizes[0] = (int64_t)N.Li.size() + n;
    sizes[1] = (int64_t)N.Ui.size() + n;
    sizes[2] = (int64_t)N.Offi.size();
    sizes[3] = S.nblocks;
    if (!Lp) return GOX_OK;
    int nz = 0;
    for (int k = 0; k < n; k++) {
      Lp[k] = nz;
      Li[nz] = k; Lx[nz] = 1.0; nz++;
      for (int p = N.Lp[k]; p < N.Lp[k + 1]; p++) { Li[nz] = N.Li[p]; Lx[nz] = N.Lx[p]; nz++; }
    }
    Lp[n] = nz;
    nz = 0;
    for (int k = 0; k < n; k++) {
      Up[k] = nz;
      for (int p = N.Up[k]; p < N.Up[k + 1]; p++) { Ui[nz] = N.Ui[p]; Ux[nz] = N.Ux[p]; nz++; }
      Ui[nz] = k; Ux[nz] = N.Udiag[k]; nz++;
    }
    Up[n] = nz;
    for (int k = 0; k <= n; k++) Fp[k] = N.Offp[k];
    for (size_t p = 0; p < N.Offi.size(); p++) { Fi[p] = N.Offi[p]; Fx[p] = N.Offx[p]; }
    for (int k = 0; k < n; k++) { P[k] = N.Pnum[k]; Q[k] = S.Q[k]; }
    for (int b = 0; b <= S.nblocks; b++) R[b] = S.R[b];
    return GOX_OK;
  });
}

int gox_topo_register(int32_t n_bus, const int32_t* yp, const int32_t* yi, const double* yre,
                      const double* yim, const int32_t* bus_type, gox_topo** out) {
  if (!out) return GOX_E_INVALID;
  *out = nullptr;
  if (n_bus <= 0 || !yp || !yi || !yre || !yim || !bus_type) return GOX_E_INVALID;
  return guard_impl([&]() -> int {
    if (yp[0] != 0) return GOX_E_INVALID;
    for (int i = 0; i < n_bus; i++) {
      if (yp[i] > yp[i + 1]) return GOX_E_INVALID;
      if (bus_type[i] < 1 || bus_type[i] > 3) return GOX_E_INVALID;
      for (int p = yp[i]; p < yp[i + 1]; p++) {
        if (yi[p] < 0 || yi[p] >= n_bus) return GOX_E_INVALID;
        if (p > yp[i] && yi[p] <= yi[p - 1]) return GOX_E_INVALID;  // sorted, no duplicates
      }
    }
    std::unique_ptr<gox_topo> t(new gox_topo());
    t->n_bus = n_bus;
    int nnz = yp[n_bus];
    t->yp.assign(yp, yp + n_bus + 1);
    t->yi.assign(yi, yi + nnz);
    t->yre.assign(yre, yre + nnz);
    t->yim.assign(yim, yim + nnz);
    t->bus_type.assign(bus_type, bus_type + n_bus);
    t->jac = jac_analyze(n_bus, yp, yi, bus_type);
    t->csc = build_csc(t->jac.n_u, t->jac.nnz(), t->jac.rows.data(), t->jac.cols.data());
    t->sym = klu_analyze(t->jac.n_u, t->csc.p.data(), t->csc.i.data());
    cudaGetDevice(&t->device);
    *out = t.release();
    return GOX_OK;
  });
}

int gox_topo_reset(gox_topo* t) {
  if (!t) return GOX_E_INVALID;
  t->twin.reset();
  t->factored = false;
  t->uploaded = false;
  t->num = Numeric();
  t->sc = Schedule();
  t->tune[0] = gox_topo::Tuning();
  t->tune[1] = gox_topo::Tuning();
  return GOX_OK;
}

void gox_topo_destroy(gox_topo* t) { delete t; }

static int check_batch_args(gox_topo* t, int B, const void* p, const void* q, const void* vm,
                            const void* va, int v_stride, double tol, int max_iter,
                            int precision, const void* vo, const void* ao, const void* it,
                            const void* st, const void* mm, const int32_t* o_slot,
                            const double* o_dre, const double* o_dim) {
  if (!t || B < 0 || max_iter < 0 || !(tol >= 0)) return GOX_E_INVALID;
  if (B == 0) return GOX_OK;
  if (!p || !q || !vm || !va || !vo || !ao || !it || !st || !mm) return GOX_E_INVALID;
  if (v_stride != 0 && v_stride != t->n_bus) return GOX_E_INVALID;
  if (precision != GOX_PRECISION_FP64 && precision != GOX_PRECISION_MIXED) return GOX_E_INVALID;
  if (o_slot && (!o_dre || !o_dim)) return GOX_E_INVALID;
  return 1;
}


int gox_batch_solve_device(gox_topo* t, int32_t B, const double* p_spec, const double* q_spec,
                           const double* vm0, const double* va0, int32_t v_stride,
                           const int32_t* o_slot, const double* o_dre, const double* o_dim,
                           double tol, int32_t max_iter, int32_t precision, double* vm_out,
                           double* va_out, int32_t* iterations, int32_t* status,
                           double* max_mismatch, double* history, void* stream) {
  int c = check_batch_args(t, B, p_spec, q_spec, vm0, va0, v_stride, tol, max_iter, precision,
                           vm_out, va_out, iterations, status, max_mismatch, o_slot, o_dre, o_dim);
  if (c <= 0) return c;
  if (int r = require_device()) return r;
  return guard_impl([&]() -> int {
    cudaStream_t st = (cudaStream_t)stream;
    AllocStreamScope alloc_scope(st);
    if (max_iter == 0) return GOX_E_INVALID;
    return batch_split(t, B, p_spec, q_spec, vm0, va0, v_stride, o_slot, o_dre, o_dim, tol,
                       max_iter, precision, vm_out, va_out, iterations, status, max_mismatch,
                       history, st, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
  });
}

int gox_batch_solve(gox_topo* t, int32_t B, const double* p_spec, const double* q_spec,
                    const double* vm0, const double* va0, int32_t v_stride,
                    const int32_t* o_slot, const double* o_dre, const double* o_dim, double tol,
                    int32_t max_iter, int32_t precision, double* vm_out, double* va_out,
                    int32_t* iterations, int32_t* status, double* max_mismatch,
                    double* history) {
  int c = check_batch_args(t, B, p_spec, q_spec, vm0, va0, v_stride, tol, max_iter, precision,
                           vm_out, va_out, iterations, status, max_mismatch, o_slot, o_dre, o_dim);
  if (c <= 0) return c;
  if (max_iter == 0) {
    std::vector<int> none;
    host_only_result(t, B, p_spec, q_spec, vm0, va0, v_stride, o_slot, o_dre, o_dim, tol, 0,
                     vm_out, va_out, iterations, status, max_mismatch, history, none);
    return GOX_OK;
  }
  if (int r = require_device()) return r;
  return guard_impl([&]() -> int {
    const int n = t->n_bus;
    cudaStream_t st = thread_stream();
    AllocStreamScope alloc_scope(st);
    const size_t bn = (size_t)B * n, nv = (size_t)(v_stride ? B : 1) * n;
    // device copies of the host arrays, kept by the topology between calls
    IoStage& io = t->io;
    DevMem &dp = io.p, &dq = io.q, &dvm = io.vm, &dva = io.va, &dovm = io.ovm, &dova = io.ova,
           &dit = io.it, &dst = io.st, &dmm = io.mm, &dh = io.h, &dsl = io.sl, &dre = io.dre,
           &dim = io.dim;
    dp.ensure(bn * 8); dq.ensure(bn * 8); dvm.ensure(nv * 8); dva.ensure(nv * 8);
    dovm.ensure(bn * 8); dova.ensure(bn * 8); dit.ensure((size_t)B * 4); dst.ensure((size_t)B * 4);
    dmm.ensure((size_t)B * 8);
    if (history) dh.ensure((size_t)B * max_iter * 8);
    GOX_CK(cudaMemcpyAsync(dp.p, p_spec, bn * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(dq.p, q_spec, bn * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(dvm.p, vm0, nv * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(dva.p, va0, nv * 8, cudaMemcpyHostToDevice, st));
    if (o_slot) {
      dsl.ensure((size_t)B * 16); dre.ensure((size_t)B * 32); dim.ensure((size_t)B * 32);
      GOX_CK(cudaMemcpyAsync(dsl.p, o_slot, (size_t)B * 16, cudaMemcpyHostToDevice, st));
      GOX_CK(cudaMemcpyAsync(dre.p, o_dre, (size_t)B * 32, cudaMemcpyHostToDevice, st));
      GOX_CK(cudaMemcpyAsync(dim.p, o_dim, (size_t)B * 32, cudaMemcpyHostToDevice, st));
    }
    int r = batch_split(t, B, dp.as<double>(), dq.as<double>(), dvm.as<double>(),
                         dva.as<double>(), v_stride, o_slot ? dsl.as<int32_t>() : nullptr,
                         o_slot ? dre.as<double>() : nullptr, o_slot ? dim.as<double>() : nullptr,
                         tol, max_iter, precision, dovm.as<double>(), dova.as<double>(),
                         dit.as<int32_t>(), dst.as<int32_t>(), dmm.as<double>(),
                         history ? dh.as<double>() : nullptr, st, p_spec, q_spec, vm0, va0,
                         o_slot, o_dre, o_dim);
    if (r != GOX_OK) return r;
    GOX_CK(cudaMemcpyAsync(vm_out, dovm.p, bn * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(va_out, dova.p, bn * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(iterations, dit.p, (size_t)B * 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(status, dst.p, (size_t)B * 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(max_mismatch, dmm.p, (size_t)B * 8, cudaMemcpyDeviceToHost, st));
    if (history)
      GOX_CK(cudaMemcpyAsync(history, dh.p, (size_t)B * max_iter * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    return GOX_OK;
  });
}

int gox_multi_solve(int32_t n_topo, gox_topo* const* topos, const int32_t* batch,
                    const double* const* p_spec, const double* const* q_spec,
                    const double* const* vm0, const double* const* va0, const int32_t* v_stride,
                    double tol, int32_t max_iter, int32_t precision, double* const* vm_out,
                    double* const* va_out, int32_t* const* iterations, int32_t* const* status,
                    double* const* max_mismatch) {
  if (n_topo < 0 || (n_topo > 0 && (!topos || !batch || !p_spec || !q_spec || !vm0 || !va0 ||
                                    !v_stride || !vm_out || !va_out || !iterations || !status ||
                                    !max_mismatch)))
    return GOX_E_INVALID;
  if (max_iter <= 0) return GOX_E_INVALID;
  std::vector<int> jobs;
  for (int j = 0; j < n_topo; j++) {
    gox_topo* t = topos[j];
    int c = check_batch_args(t, batch[j], p_spec[j], q_spec[j], vm0[j], va0[j], v_stride[j], tol,
                             max_iter, precision, vm_out[j], va_out[j], iterations[j], status[j],
                             max_mismatch[j], nullptr, nullptr, nullptr);
    if (c < 0) return c;
    if (!t->zip.empty()) return GOX_E_INVALID;  // ZIP terms: one gox_batch_solve per topology
    for (int k : jobs)
      if (topos[k] == t) return GOX_E_INVALID;  // a topology's buffers serve one batch
    if (c > 0) jobs.push_back(j);
  }
  if (jobs.empty()) return GOX_OK;
  if (int r = require_device()) return r;
  // each job's set-up and results on up to 8 host threads (each its own
  // stream), the solve itself on the calling thread's stream
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GOX_E_CUDA;
  auto parallel = [&](size_t n, const std::function<int(size_t)>& fn) -> int {
    const size_t nt = std::min<size_t>(n, 8);
    std::vector<int> rc(nt, GOX_OK);
    std::vector<std::thread> th;
    for (size_t w = 0; w < nt; w++)
      th.emplace_back([&, w] {
        rc[w] = guard_impl([&]() -> int {
          GOX_CK(cudaSetDevice(dev));
          cudaStream_t ws = thread_stream();
          AllocStreamScope scope(ws);
          for (size_t k = w; k < n; k += nt)
            if (int r = fn(k)) return r;
          return GOX_OK;
        });
      });
    for (auto& x : th) x.join();
    for (int r : rc)
      if (r != GOX_OK) return r;
    return GOX_OK;
  };
  std::vector<BatchRun> all(jobs.size());
  int rc = parallel(jobs.size(), [&](size_t k) -> int {
    const int j = jobs[k];
    gox_topo* t = topos[j];
    cudaStream_t ws = thread_stream();
    const int B = batch[j], n = t->n_bus;
    const size_t bn = (size_t)B * n, nv = (size_t)(v_stride[j] ? B : 1) * n;
    IoStage& io = t->io;
    io.p.ensure(bn * 8); io.q.ensure(bn * 8); io.vm.ensure(nv * 8); io.va.ensure(nv * 8);
    io.ovm.ensure(bn * 8); io.ova.ensure(bn * 8); io.it.ensure((size_t)B * 4);
    io.st.ensure((size_t)B * 4); io.mm.ensure((size_t)B * 8);
    GOX_CK(cudaMemcpyAsync(io.p.p, p_spec[j], bn * 8, cudaMemcpyHostToDevice, ws));
    GOX_CK(cudaMemcpyAsync(io.q.p, q_spec[j], bn * 8, cudaMemcpyHostToDevice, ws));
    GOX_CK(cudaMemcpyAsync(io.vm.p, vm0[j], nv * 8, cudaMemcpyHostToDevice, ws));
    GOX_CK(cudaMemcpyAsync(io.va.p, va0[j], nv * 8, cudaMemcpyHostToDevice, ws));
    const int r = batch_prepare(
        t, B, io.p.as<double>(), io.q.as<double>(), io.vm.as<double>(), io.va.as<double>(),
        v_stride[j], nullptr, nullptr, nullptr, tol, max_iter, precision, io.ovm.as<double>(),
        io.ova.as<double>(), io.it.as<int32_t>(), io.st.as<int32_t>(), io.mm.as<double>(),
        nullptr, ws, p_spec[j], q_spec[j], vm0[j], va0[j], nullptr, nullptr, nullptr, all[k]);
    GOX_CK(cudaStreamSynchronize(ws));  // set up before the solve's stream uses it
    return r;
  });
  if (rc != GOX_OK) return rc;
  std::vector<gox_topo*> ts;
  std::vector<BatchRun> runs;
  std::vector<int> of;  // solved job -> argument index
  for (size_t k = 0; k < jobs.size(); k++)
    if (!all[k].resolved) {
      ts.push_back(topos[jobs[k]]);
      runs.push_back(all[k]);
      of.push_back(jobs[k]);
    }
  int64_t launches = 0;
  if (!ts.empty()) {
    rc = guard_impl([&]() -> int {
      cudaStream_t st = thread_stream();
      AllocStreamScope alloc_scope(st);
      // the persistent kernel needs every schedule's forward substitution
      // fused (no off-diagonal BTF blocks: no separate solve launch)
      bool persistent = g_multi_persistent.load() != 0;
      const int pi = precision == GOX_PRECISION_FP64 ? 1 : 0;
      for (gox_topo* t : ts) persistent = persistent && t->sc.fuse_fwd && persist_plan(t, pi);
      if (persistent) {
        if (precision == GOX_PRECISION_FP64) run_persistent<double>(ts, runs, max_iter, st, launches);
        else run_persistent<float>(ts, runs, max_iter, st, launches);
      } else {
        if (precision == GOX_PRECISION_FP64) run_multi<double>(ts, runs, max_iter, st, launches);
        else run_multi<float>(ts, runs, max_iter, st, launches);
      }
      return GOX_OK;
    });
    if (rc != GOX_OK) return rc;
  }
  std::vector<int> run_of(n_topo, -1);
  for (size_t k = 0; k < of.size(); k++) run_of[of[k]] = (int)k;
  return parallel(jobs.size(), [&](size_t k) -> int {
    const int j = jobs[k];
    gox_topo* t = topos[j];
    cudaStream_t ws = thread_stream();
    IoStage& io = t->io;
    const int B = batch[j];
    if (run_of[j] >= 0) {
      const int r = batch_finish(
          t, B, io.p.as<double>(), io.q.as<double>(), io.vm.as<double>(), io.va.as<double>(),
          v_stride[j], nullptr, nullptr, nullptr, tol, max_iter, precision, io.ovm.as<double>(),
          io.ova.as<double>(), io.it.as<int32_t>(), io.st.as<int32_t>(), io.mm.as<double>(),
          nullptr, ws, p_spec[j], q_spec[j], vm0[j], va0[j], nullptr, nullptr, nullptr,
          runs[run_of[j]]);
      if (r != GOX_OK) return r;
      t->launches += launches / (int64_t)ts.size();
    }
    const size_t bn = (size_t)B * t->n_bus;
    GOX_CK(cudaMemcpyAsync(vm_out[j], io.ovm.p, bn * 8, cudaMemcpyDeviceToHost, ws));
    GOX_CK(cudaMemcpyAsync(va_out[j], io.ova.p, bn * 8, cudaMemcpyDeviceToHost, ws));
    GOX_CK(cudaMemcpyAsync(iterations[j], io.it.p, (size_t)B * 4, cudaMemcpyDeviceToHost, ws));
    GOX_CK(cudaMemcpyAsync(status[j], io.st.p, (size_t)B * 4, cudaMemcpyDeviceToHost, ws));
    GOX_CK(cudaMemcpyAsync(max_mismatch[j], io.mm.p, (size_t)B * 8, cudaMemcpyDeviceToHost, ws));
    GOX_CK(cudaStreamSynchronize(ws));
    return GOX_OK;
  });
}

int gox_batch_solve_scaled(gox_topo* t, int32_t B, const double* scales, const double* p_base,
                           const double* q_base, const double* vm0, const double* va0, double tol,
                           int32_t max_iter, int32_t precision, double* vm_out, double* va_out,
                           int32_t* iterations, int32_t* status, double* max_mismatch,
                           double* history) {
  int c = check_batch_args(t, B, p_base, q_base, vm0, va0, 0, tol, max_iter, precision, vm_out,
                           va_out, iterations, status, max_mismatch, nullptr, nullptr, nullptr);
  if (c <= 0) return c;
  if (!scales) return GOX_E_INVALID;
  const int n = t->n_bus;
  if (max_iter == 0) {
    std::vector<double> hp((size_t)B * n), hq((size_t)B * n);
    for (int s = 0; s < B; s++)
      for (int i = 0; i < n; i++) {
        hp[(size_t)s * n + i] = p_base[i] * scales[s];
        hq[(size_t)s * n + i] = q_base[i] * scales[s];
      }
    std::vector<int> none;
    host_only_result(t, B, hp.data(), hq.data(), vm0, va0, 0, nullptr, nullptr, nullptr, tol, 0,
                     vm_out, va_out, iterations, status, max_mismatch, history, none);
    return GOX_OK;
  }
  if (int r = require_device()) return r;
  return guard_impl([&]() -> int {
    cudaStream_t st = thread_stream();
    AllocStreamScope alloc_scope(st);
    const size_t bn = (size_t)B * n;
    IoStage& io = t->io;
    io.p.ensure(bn * 8); io.q.ensure(bn * 8); io.vm.ensure((size_t)n * 8); io.va.ensure((size_t)n * 8);
    io.pb.ensure((size_t)n * 8); io.qb.ensure((size_t)n * 8); io.sc.ensure((size_t)B * 8);
    io.ovm.ensure(bn * 8); io.ova.ensure(bn * 8); io.it.ensure((size_t)B * 4);
    io.st.ensure((size_t)B * 4); io.mm.ensure((size_t)B * 8);
    if (history) io.h.ensure((size_t)B * max_iter * 8);
    GOX_CK(cudaMemcpyAsync(io.pb.p, p_base, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(io.qb.p, q_base, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(io.sc.p, scales, (size_t)B * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(io.vm.p, vm0, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(io.va.p, va0, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    k_scale_rows<<<grid1d(bn), 256, 0, st>>>(io.pb.as<double>(), io.qb.as<double>(),
                                             io.sc.as<double>(), B, n, io.p.as<double>(),
                                             io.q.as<double>());
    GOX_CK(cudaGetLastError());
    // the pivot search (first call) reads the scaled injections back from the device
    int r = batch_device(t, B, io.p.as<double>(), io.q.as<double>(), io.vm.as<double>(),
                         io.va.as<double>(), 0, nullptr, nullptr, nullptr, tol, max_iter, precision,
                         io.ovm.as<double>(), io.ova.as<double>(), io.it.as<int32_t>(),
                         io.st.as<int32_t>(), io.mm.as<double>(),
                         history ? io.h.as<double>() : nullptr, st, nullptr, nullptr, nullptr,
                         nullptr, nullptr, nullptr, nullptr);
    t->launches += 1;
    if (r != GOX_OK) return r;
    GOX_CK(cudaMemcpyAsync(vm_out, io.ovm.p, bn * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(va_out, io.ova.p, bn * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(iterations, io.it.p, (size_t)B * 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(status, io.st.p, (size_t)B * 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(max_mismatch, io.mm.p, (size_t)B * 8, cudaMemcpyDeviceToHost, st));
    if (history)
      GOX_CK(cudaMemcpyAsync(history, io.h.p, (size_t)B * max_iter * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    return GOX_OK;
  });
}

int gox_batch_solve_qlim(gox_topo* t, int32_t B, const double* p_spec, const double* q_spec,
                         const double* vm0, const double* va0, int32_t v_stride,
                         const double* q_min, const double* q_max, double tol, int32_t max_iter,
                         int32_t max_outer, int32_t precision, double* vm_out, double* va_out,
                         int32_t* iterations, int32_t* status, double* max_mismatch,
                         int32_t* n_switched, uint8_t* switched, int32_t* stabilized) {
  int c = check_batch_args(t, B, p_spec, q_spec, vm0, va0, v_stride, tol, max_iter, precision,
                           vm_out, va_out, iterations, status, max_mismatch, nullptr, nullptr,
                           nullptr);
  if (c <= 0) return c;
  if (!q_min || !q_max || !n_switched || !stabilized || max_outer < 1 || max_iter < 1)
    return GOX_E_INVALID;
  if (int r = require_device()) return r;
  return guard_impl([&]() -> int {
    const int n = t->n_bus;
    cudaStream_t st = thread_stream();
    AllocStreamScope alloc_scope(st);
    const size_t bn = (size_t)B * n, nv = (size_t)(v_stride ? B : 1) * n;
    // the batch's state on the device: injections (q pinned as buses switch), V
    DevMem dp, dq, dv0m, dv0a, dvm, dva, dit, dst, dmm;
    dp.ensure(bn * 8); dq.ensure(bn * 8); dv0m.ensure(nv * 8); dv0a.ensure(nv * 8);
    dvm.ensure(bn * 8); dva.ensure(bn * 8);
    dit.ensure((size_t)B * 4); dst.ensure((size_t)B * 4); dmm.ensure((size_t)B * 8);
    GOX_CK(cudaMemcpyAsync(dp.p, p_spec, bn * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(dq.p, q_spec, bn * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(dv0m.p, vm0, nv * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(dv0a.p, va0, nv * 8, cudaMemcpyHostToDevice, st));
    // pass 1: every scenario on the topology as given (its own start rule)
    int r = batch_device(t, B, dp.as<double>(), dq.as<double>(), dv0m.as<double>(),
                         dv0a.as<double>(), v_stride, nullptr, nullptr, nullptr, tol, max_iter,
                         precision, dvm.as<double>(), dva.as<double>(), dit.as<int32_t>(),
                         dst.as<int32_t>(), dmm.as<double>(), nullptr, st, p_spec, q_spec, vm0,
                         va0, nullptr, nullptr, nullptr);
    if (r != GOX_OK) return r;
    std::vector<int32_t> pv;  // the PV buses of the given topology
    for (int i = 0; i < n; i++)
      if (t->bus_type[i] == 2) pv.push_back(i);
    const int npv = (int)pv.size();
    std::vector<std::vector<int32_t>> sw(B);  // switched buses per scenario, sorted
    std::vector<uint8_t> done(B, 0);
    std::vector<int32_t> hst(B);
    std::vector<double> hq((size_t)B * std::max(npv, 1));
    DevMem dyp, dyi, dyre, dyim, dpv, dqc, dsb, dval;
    upload(dyp, t->yp); upload(dyi, t->yi); upload(dyre, t->yre); upload(dyim, t->yim);
    upload(dpv, pv);
    dqc.ensure((size_t)B * std::max(npv, 1) * 8);
    for (int s = 0; s < B; s++) stabilized[s] = 1;
    for (int pass = 1;; pass++) {
      GOX_CK(cudaMemcpyAsync(hst.data(), dst.p, (size_t)B * 4, cudaMemcpyDeviceToHost, st));
      if (npv > 0) {
        k_qcalc<<<grid1d((size_t)B * npv), 256, 0, st>>>(
            B, n, dyp.as<int32_t>(), dyi.as<int32_t>(), dyre.as<double>(), dyim.as<double>(),
            dvm.as<double>(), dva.as<double>(), dpv.as<int32_t>(), npv, dqc.as<double>());
        GOX_CK(cudaGetLastError());
        GOX_CK(cudaMemcpyAsync(hq.data(), dqc.p, (size_t)B * npv * 8, cudaMemcpyDeviceToHost, st));
      }
      GOX_CK(cudaStreamSynchronize(st));
      // PV -> PQ switching of every settled scenario, pinning Q at the violated limit
      std::vector<int32_t> pin_sb;
      std::vector<double> pin_val;
      std::map<std::vector<int32_t>, std::vector<int32_t>> groups;
      for (int s = 0; s < B; s++) {
        if (done[s]) continue;
        if (hst[s] != GOX_CONVERGED) {  // not settled: that pass's report stands
          done[s] = 1;
          continue;
        }
        bool any = false;
        std::vector<int32_t>& w = sw[s];
        const std::vector<int32_t> before = w;
        for (int k = 0; k < npv; k++) {
          const int b = pv[k];
          if (std::binary_search(before.begin(), before.end(), b)) continue;  // already PQ
          const double qc = hq[(size_t)s * npv + k];
          double lim;
          if (qc < q_min[b]) lim = q_min[b];
          else if (qc > q_max[b]) lim = q_max[b];
          else continue;
          pin_sb.insert(pin_sb.end(), {s, b});
          pin_val.push_back(lim);
          w.push_back(b);
          any = true;
        }
        if (!any) {
          done[s] = 1;
          continue;
        }
        std::sort(w.begin(), w.end());
        if (pass == max_outer) {  // outer budget spent: the last solve's report, not stabilized
          done[s] = 1;
          stabilized[s] = 0;
          continue;
        }
        groups[w].push_back(s);
      }
      if (!pin_val.empty()) {
        upload(dsb, pin_sb);
        upload(dval, pin_val);
        const int m = (int)pin_val.size();
        k_pin<<<(m + 255) / 256, 256, 0, st>>>(m, dsb.as<int32_t>(), dval.as<double>(), n,
                                               dq.as<double>());
        GOX_CK(cudaGetLastError());
      }
      if (groups.empty()) break;
      // re-solve each group on its variant, warm started from its state: the
      // variants are built here (host analysis, in order), then the groups run
      // concurrently, up to kQlimWorkers host threads with a stream and staging
      // buffers each, on disjoint rows of the batch state
      std::vector<std::pair<gox_topo*, const std::vector<int32_t>*>> jobs;
      for (auto& gk : groups) {
        std::vector<int32_t> changes(gk.first.size());
        for (size_t k = 0; k < changes.size(); k++) changes[k] = gk.first[k] * 4 + 1;  // PV -> PQ
        jobs.emplace_back(topo_variant(t, changes), &gk.second);
      }
      GOX_CK(cudaStreamSynchronize(st));  // the pins are in dq
      std::atomic<int> next{0}, err{GOX_OK};
      auto work = [&]() {
        const int rc = guard_impl([&]() -> int {
          GOX_CK(cudaSetDevice(t->device));
          cudaStream_t ws = nullptr;
          GOX_CK(cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking));
          struct WorkStream {
            cudaStream_t s;
            ~WorkStream() { cudaStreamDestroy(s); }
          } wsg{ws};
          AllocStreamScope alloc_scope(ws);
          DevMem dix, sp, sq, svm, sva, ovm, ova, oit, ost, omm;
          for (int j = next++; j < (int)jobs.size() && err.load() == GOX_OK; j = next++) {
            gox_topo* v = jobs[j].first;
            const std::vector<int32_t>& idx = *jobs[j].second;
            const int Bg = (int)idx.size();
            const size_t rows = (size_t)Bg * n;
            upload(dix, idx);
            const int32_t* ix = dix.as<int32_t>();
            sp.ensure(rows * 8); sq.ensure(rows * 8); svm.ensure(rows * 8); sva.ensure(rows * 8);
            ovm.ensure(rows * 8); ova.ensure(rows * 8);
            oit.ensure((size_t)Bg * 4); ost.ensure((size_t)Bg * 4); omm.ensure((size_t)Bg * 8);
            k_take_rows<double><<<grid1d(rows), 256, 0, ws>>>(dp.as<double>(), n, ix, Bg, sp.as<double>());
            k_take_rows<double><<<grid1d(rows), 256, 0, ws>>>(dq.as<double>(), n, ix, Bg, sq.as<double>());
            k_take_rows<double><<<grid1d(rows), 256, 0, ws>>>(dvm.as<double>(), n, ix, Bg, svm.as<double>());
            k_take_rows<double><<<grid1d(rows), 256, 0, ws>>>(dva.as<double>(), n, ix, Bg, sva.as<double>());
            const int rg = batch_device(v, Bg, sp.as<double>(), sq.as<double>(), svm.as<double>(),
                                        sva.as<double>(), n, nullptr, nullptr, nullptr, tol, max_iter,
                                        precision, ovm.as<double>(), ova.as<double>(),
                                        oit.as<int32_t>(), ost.as<int32_t>(), omm.as<double>(), nullptr,
                                        ws, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
            if (rg != GOX_OK) return rg;
            k_put_rows<double><<<grid1d(rows), 256, 0, ws>>>(ovm.as<double>(), n, ix, Bg, dvm.as<double>());
            k_put_rows<double><<<grid1d(rows), 256, 0, ws>>>(ova.as<double>(), n, ix, Bg, dva.as<double>());
            k_put_rows<int32_t><<<grid1d(Bg), 256, 0, ws>>>(oit.as<int32_t>(), 1, ix, Bg, dit.as<int32_t>());
            k_put_rows<int32_t><<<grid1d(Bg), 256, 0, ws>>>(ost.as<int32_t>(), 1, ix, Bg, dst.as<int32_t>());
            k_put_rows<double><<<grid1d(Bg), 256, 0, ws>>>(omm.as<double>(), 1, ix, Bg, dmm.as<double>());
            GOX_CK(cudaGetLastError());
            GOX_CK(cudaStreamSynchronize(ws));  // the staging buffers are reused by the next group
          }
          return GOX_OK;
        });
        if (rc != GOX_OK) {
          int ok = GOX_OK;
          err.compare_exchange_strong(ok, rc);
        }
      };
      const int nw = std::min<int>(kQlimWorkers, (int)jobs.size());
      std::vector<std::thread> pool;
      for (int w = 1; w < nw; w++) pool.emplace_back(work);
      work();
      for (auto& th : pool) th.join();
      if (err.load() != GOX_OK) return err.load();
    }
    GOX_CK(cudaMemcpyAsync(vm_out, dvm.p, bn * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(va_out, dva.p, bn * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(iterations, dit.p, (size_t)B * 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(status, dst.p, (size_t)B * 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(max_mismatch, dmm.p, (size_t)B * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    for (int s = 0; s < B; s++) n_switched[s] = (int32_t)sw[s].size();
    if (switched) {
      std::fill(switched, switched + bn, (uint8_t)0);
      for (int s = 0; s < B; s++)
        for (int b : sw[s]) switched[(size_t)s * n + b] = 1;
    }
    return GOX_OK;
  });
}

int gox_outage_islands(gox_topo* t, int32_t B, const int32_t* out_slot, const double* out_dre,
                       const double* out_dim, int32_t* n_islands, int32_t* island_of,
                       int32_t* verdict) {
  if (!t || B < 0 || !out_slot || !out_dre || !out_dim || !n_islands) return GOX_E_INVALID;
  return guard_impl([&]() -> int {
    const int n = t->n_bus;
    if (t->base_label.empty()) t->base_label = components_without(t, -1, -1);
    std::vector<int32_t> pinned;
    for (int s = 0; s < B; s++) {
      const std::vector<int32_t>& split =
          outage_split(t, out_slot + 4 * s, out_dre + 4 * s, out_dim + 4 * s, &pinned);
      const std::vector<int32_t>& label = split.empty() ? t->base_label : split;
      const int nc = 1 + *std::max_element(label.begin(), label.end());
      n_islands[s] = nc;
      std::vector<int32_t> slacks(nc, 0);
      for (int i = 0; i < n; i++)
        if (t->bus_type[i] == 3) slacks[label[i]]++;
      for (int i = 0; i < n; i++) {
        if (island_of) island_of[(size_t)s * n + i] = label[i];
        if (verdict) {
          const int k = slacks[label[i]];
          verdict[(size_t)s * n + i] = k == 1 ? GOX_ISLAND_SOLVABLE
                                              : (k == 0 ? GOX_ISLAND_NO_REFERENCE : GOX_ISLAND_AMBIGUOUS);
        }
      }
    }
    return GOX_OK;
  });
}

int gox_topo_prepare(gox_topo* t, int32_t B, const double* p_spec, const double* q_spec,
                     const double* vm0, const double* va0, int32_t v_stride,
                     const int32_t* o_slot, const double* o_dre, const double* o_dim, double tol) {
  if (!t || B <= 0 || !p_spec || !q_spec || !vm0 || !va0 || !(tol >= 0)) return GOX_E_INVALID;
  if (v_stride != 0 && v_stride != t->n_bus) return GOX_E_INVALID;
  if (o_slot && (!o_dre || !o_dim)) return GOX_E_INVALID;
  return guard_impl([&]() -> int {
    if (t->factored) return GOX_OK;
    std::vector<int> first_singular;
    int s = fix_pivots(t, B, p_spec, q_spec, vm0, va0, v_stride, o_slot, o_dre, o_dim, tol,
                       first_singular);
    return s < 0 ? GOX_SINGULAR : GOX_OK;
  });
}

// Host mirror of k_refactor (+ fused forward) and k_solve for one scenario:
// same batches, stage positions, phases and term lists, FP64.
int gox_topo_emulate_step(const gox_topo* t, const double* jac_vals, const double* rhs,
                          double* dx) {
  if (!t || !t->factored || !jac_vals || !rhs || !dx) return GOX_E_INVALID;
  return guard_impl([&]() -> int {
    const Schedule& sc = t->sc;
    const int n = sc.n_u;
    std::vector<double> lu(sc.n_slots, 0.0), off(std::max(sc.n_off, 1), 0.0), X(n, 0.0),
        b(n), st(sc.max_collen);
    for (int u = 0; u < n; u++) b[t->num.Pinv[u]] = rhs[u];
    // A values in consumption order
    std::vector<double> packed(t->csc.nnz(), 0.0);
    for (int e = 0; e < t->jac.nnz(); e++) packed[t->csc.slot_of[e]] += jac_vals[e];
    bool bad = false;
    // the factor's starting image (A values, zeros at fill-in), then the
    // refactor streams of both precisions run by the host interpreter:
    // both must pass every check and give the same factor
    for (int x = 0; x < sc.n_slots; x++) lu[x] = sc.slot_a[x] >= 0 ? packed[sc.a_csc[sc.slot_a[x]]] : 0.0;
    for (int a = 0; a < sc.n_a; a++)
      if (sc.a_dst[a] < 0) off[-sc.a_dst[a] - 1] = packed[sc.a_csc[a]];
    std::vector<double> lu64 = lu, X64;
    bool sing32 = false, sing64 = false;
    std::string e32 = run_stream_host(sc, t->s32, lu, b, X, sing32);
    if (!e32.empty()) throw std::runtime_error("FP32 refactor stream: " + e32);
    std::string e64 = run_stream_host(sc, t->s64, lu64, b, X64, sing64);
    if (!e64.empty()) throw std::runtime_error("FP64 refactor stream: " + e64);
    for (int x = 0; x < sc.n_slots; x++)
      if (!(lu[x] == lu64[x]) && !(std::isnan(lu[x]) && std::isnan(lu64[x])))
        throw std::runtime_error("the two refactor streams disagree");
    bad = sing32;
    if (t->s32.has_bwd != t->s64.has_bwd) throw std::runtime_error("stream plans disagree");
    for (int x = 0; x < n && t->s32.has_bwd; x++)
      if (!(X[x] == X64[x]) && !(std::isnan(X[x]) && std::isnan(X64[x])))
        throw std::runtime_error("the two streams' substitutions disagree");
    for (int ph = 0; ph < sc.n_phases && !t->s32.has_bwd; ph++) {
      for (int q = sc.ph_ptr[ph]; q < sc.ph_ptr[ph + 1]; q++) {
        const int k = sc.ph_rows[q];
        if (sc.ph_kind[ph] == 0) {
          double v = b[k];
          for (int tt = sc.fw_ptr[k]; tt < sc.fw_ptr[k + 1]; tt++) {
            const int sl = sc.fw_slot[tt];
            v -= (sl >= 0 ? lu[sl] : off[-sl - 1]) * X[sc.fw_col[tt]];
          }
          X[k] = v;
        } else {
          double v = X[k];
          for (int tt = sc.bw_ptr[k]; tt < sc.bw_ptr[k + 1]; tt++) v -= lu[sc.bw_slot[tt]] * X[sc.bw_col[tt]];
          v = v / lu[sc.diag_slot[k]];
          if (!std::isfinite(v)) bad = true;
          X[k] = v;
        }
      }
    }
    for (int k = 0; k < n; k++) dx[t->sym.Q[k]] = X[k];
    return bad ? GOX_SINGULAR : GOX_OK;
  });
}

}  // extern "C"

// One mismatch, fill and refactor of the batch path at given voltages, with
// the Jacobian image (after the fill) and the factor (after the refactor)
// read back: the per-entry view the parity tests compare with the oracle.
template <typename T>
static void factor_values_run(gox_topo* t, const BatchDev& D, int B, cudaStream_t st,
                              double* jac_vals, double* lu_vals) {
  const SchedDev& S = t->dsched.d;
  const Schedule& sc = t->sc;
  const size_t nl = (size_t)D.G * S.n_slots * 32, no = (size_t)D.G * S.n_off * 32;
  std::vector<T> img(nl), offv(no);
  GOX_CK(cudaMemsetAsync(D.nactive, 0, sizeof(int32_t), st));
  Iter<T>::mismatch(S, D, 0, 0, false, st);
  Iter<T>::fill(S, D, false, st);
  if (jac_vals) {
    GOX_CK(cudaMemcpyAsync(img.data(), D.lu, nl * sizeof(T), cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(offv.data(), D.off, no * sizeof(T), cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    // emission entry e -> CSC slot -> A entry (consumption order) -> LU slot
    // or off-diagonal entry of the image
    std::vector<int32_t> a_of_csc(t->csc.nnz(), -1), slot_of_a(sc.n_a, -1);
    for (int a = 0; a < sc.n_a; a++) a_of_csc[sc.a_csc[a]] = a;
    for (int x = 0; x < sc.n_slots; x++)
      if (sc.slot_a[x] >= 0) slot_of_a[sc.slot_a[x]] = x;
    const int nj = t->jac.nnz();
    for (int e = 0; e < nj; e++) {
      const int a = a_of_csc[t->csc.slot_of[e]];
      const int x = slot_of_a[a];
      for (int sn = 0; sn < B; sn++) {
        const int g = sn / 32, l = sn % 32;
        const T v = sc.a_dst[a] >= 0 ? img[((size_t)g * S.n_slots + x) * 32 + l]
                                     : offv[((size_t)g * S.n_off + (-sc.a_dst[a] - 1)) * 32 + l];
        jac_vals[(size_t)sn * nj + e] = (double)v;
      }
    }
  }
  Iter<T>::refactor(t->dsched, D, st);
  GOX_CK(cudaGetLastError());
  if (lu_vals) {
    GOX_CK(cudaMemcpyAsync(img.data(), D.lu, nl * sizeof(T), cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    for (int sn = 0; sn < B; sn++) {
      const int g = sn / 32, l = sn % 32;
      for (int x = 0; x < S.n_slots; x++)
        lu_vals[(size_t)sn * S.n_slots + x] = (double)img[((size_t)g * S.n_slots + x) * 32 + l];
    }
  }
  GOX_CK(cudaStreamSynchronize(st));
}

extern "C" {

int gox_topo_factor_values(gox_topo* t, int32_t B, const double* p_spec, const double* q_spec,
                           const double* vm, const double* va, int32_t precision,
                           double* jac_vals, double* lu_vals) {
  if (!t || B <= 0 || !p_spec || !q_spec || !vm || !va || !t->factored) return GOX_E_INVALID;
  if (precision != GOX_PRECISION_FP64 && precision != GOX_PRECISION_MIXED) return GOX_E_INVALID;
  if (int r = require_device()) return r;
  return guard_impl([&]() -> int {
    cudaStream_t st = thread_stream();
    AllocStreamScope alloc_scope(st);
    const int n = t->n_bus, G = (B + 31) / 32;
    if (!t->uploaded) {
      t->dsched.load(t->sc, t->yp, t->yi, t->yre, t->yim);
      t->dsched.load_streams(t->s32, t->s64);
      t->uploaded = true;
    }
    t->dsched.d.zip = t->zip.empty() ? nullptr : t->dzip.as<double>();
    const SchedDev& S = t->dsched.d;
    DevBatch& DB = t->batch;
    DB.ensure(S, G, precision, 1, false);
    // tol 0: no scenario counts as converged, so every group is filled and
    // refactored
    BatchDev D = DB.view(false, false, 0.0, 0.0);
    IoStage& io = t->io;
    const size_t bn = (size_t)B * n;
    io.p.ensure(bn * 8); io.q.ensure(bn * 8); io.vm.ensure(bn * 8); io.va.ensure(bn * 8);
    GOX_CK(cudaMemcpyAsync(io.p.p, p_spec, bn * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(io.q.p, q_spec, bn * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(io.vm.p, vm, bn * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(io.va.p, va, bn * 8, cudaMemcpyHostToDevice, st));
    const size_t tot = (size_t)G * n * 32;
    k_scatter_rows<<<grid1d(tot), 256, 0, st>>>(io.p.as<double>(), B, n, n, D.psp, G);
    k_scatter_rows<<<grid1d(tot), 256, 0, st>>>(io.q.as<double>(), B, n, n, D.qsp, G);
    k_scatter_rows<<<grid1d(tot), 256, 0, st>>>(io.vm.as<double>(), B, n, n, D.vm, G);
    k_scatter_rows<<<grid1d(tot), 256, 0, st>>>(io.va.as<double>(), B, n, n, D.va, G);
    k_init_scen<<<(G * 32 + 255) / 256, 256, 0, st>>>(B, G, D.status, D.iters, D.sing,
                                                       D.piv_flag, D.maxmis, D.maxacc);
    GOX_CK(cudaMemsetAsync(DB.err.p, 0, 16, st));
    if (precision == GOX_PRECISION_FP64) factor_values_run<double>(t, D, B, st, jac_vals, lu_vals);
    else factor_values_run<float>(t, D, B, st, jac_vals, lu_vals);
    int32_t herr[2] = {0, 0};
    GOX_CK(cudaMemcpyAsync(herr, DB.err.p, 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    return herr[1] ? GOX_E_DEVICE_WAIT : GOX_OK;
  });
}

int gox_topo_pivot_solve(gox_topo* t, const double* jac_vals, const double* rhs, double* dx) {
  if (!t || !t->factored || !jac_vals || !rhs || !dx) return GOX_E_INVALID;
  if (int r = require_device()) return r;
  return guard_impl([&]() -> int {
    cudaStream_t st = thread_stream();
    AllocStreamScope alloc_scope(st);
    const Schedule& sc = t->sc;
    const int n = sc.n_u;
    if (!t->uploaded) {
      t->dsched.load(t->sc, t->yp, t->yi, t->yre, t->yim);
      t->dsched.load_streams(t->s32, t->s64);
      t->uploaded = true;
    }
    const SchedDev& S = t->dsched.d;
    DevBatch& DB = t->batch;
    DB.ensure(S, 1, GOX_PRECISION_FP64, 1, false);
    BatchDev D = DB.view(false, false, 0.0, 0.0);
    // the fill image of one group: the Jacobian in lane 0 (the other lanes
    // are unused scenarios), the right-hand side in the static pivot order
    std::vector<double> packed(t->csc.nnz(), 0.0);
    for (int e = 0; e < t->jac.nnz(); e++) packed[t->csc.slot_of[e]] += jac_vals[e];
    std::vector<double> img((size_t)S.n_slots * 32, 0.0), off((size_t)S.n_off * 32, 0.0),
        b((size_t)n * 32, 0.0), x((size_t)n * 32, 0.0);
    for (int xs = 0; xs < sc.n_slots; xs++)
      if (sc.slot_a[xs] >= 0) img[(size_t)xs * 32] = packed[sc.a_csc[sc.slot_a[xs]]];
    for (int a = 0; a < sc.n_a; a++)
      if (sc.a_dst[a] < 0) off[(size_t)(-sc.a_dst[a] - 1) * 32] = packed[sc.a_csc[a]];
    for (int u = 0; u < n; u++) b[(size_t)t->num.Pinv[u] * 32] = rhs[u];
    std::vector<int32_t> status(32, ST_UNUSED), zeros(32, 0), one(1, 1);
    status[0] = ST_RUNNING;
    GOX_CK(cudaMemcpyAsync(D.lu, img.data(), img.size() * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(D.off, off.data(), off.size() * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(D.rhs, b.data(), b.size() * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(D.status, status.data(), 128, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(D.sing, zeros.data(), 128, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(D.gact, one.data(), 4, cudaMemcpyHostToDevice, st));
    pivot_run(t, D, st);
    GOX_CK(cudaGetLastError());
    int32_t sing = 0;
    GOX_CK(cudaMemcpyAsync(x.data(), D.sol, x.size() * 8, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaMemcpyAsync(&sing, D.sing, 4, cudaMemcpyDeviceToHost, st));
    GOX_CK(cudaStreamSynchronize(st));
    for (int k = 0; k < n; k++) dx[t->sym.Q[k]] = x[(size_t)k * 32];
    return sing ? GOX_SINGULAR : GOX_OK;
  });
}

int gox_topo_stream_word(gox_topo* t, int32_t precision, int32_t warp, int32_t index,
                         int32_t value, int32_t* old_value) {
  if (!t || !t->factored || !t->uploaded) return GOX_E_INVALID;
  if (precision != GOX_PRECISION_FP64 && precision != GOX_PRECISION_MIXED) return GOX_E_INVALID;
  const Stream& s = precision == GOX_PRECISION_MIXED ? t->s32 : t->s64;
  if (warp < 0 || warp >= s.plan.nw || index < 0 ||
      (int64_t)index >= (int64_t)s.nchunks[warp] * s.plan.chunk_words)
    return GOX_E_INVALID;
  return guard_impl([&]() -> int {
    const int i = precision == GOX_PRECISION_MIXED ? 0 : 1;
    int32_t* w = t->dsched.sw[i].as<int32_t>() + (size_t)s.chunk0[warp] * s.plan.chunk_words + index;
    int32_t old = 0;
    GOX_CK(cudaDeviceSynchronize());
    GOX_CK(cudaMemcpy(&old, w, 4, cudaMemcpyDeviceToHost));
    GOX_CK(cudaMemcpy(w, &value, 4, cudaMemcpyHostToDevice));
    if (old_value) *old_value = old;
    return GOX_OK;
  });
}

int gox_set_autotune(int32_t on) {
  g_autotune.store(on ? 1 : 0);
  return GOX_OK;
}

int gox_set_refactor_sync(int32_t flags) {
  g_refactor_sync.store(flags ? 1 : 0);
  return GOX_OK;
}

int gox_set_multi_persistent(int32_t on) {
  g_multi_persistent.store(on ? 1 : 0);
  return GOX_OK;
}

int gox_set_refactor_wide(int32_t min_width) {
  if (min_width < 0) return GOX_E_INVALID;
  g_refactor_wide.store(min_width);
  return GOX_OK;
}

int gox_topo_tuning(const gox_topo* t, int32_t precision, int64_t* plan, double* table,
                    int32_t max_rows) {
  if (!t || !plan || (precision != GOX_PRECISION_FP64 && precision != GOX_PRECISION_MIXED))
    return GOX_E_INVALID;
  if (!t->factored) return GOX_E_INVALID;
  const int i = precision == GOX_PRECISION_MIXED ? 0 : 1;
  const Stream& s = i == 0 ? t->s32 : t->s64;
  const gox_topo::Tuning& TU = t->tune[i];
  plan[0] = s.plan.nw;
  plan[1] = s.plan.ring_rows;
  plan[2] = s.plan.big_rows;
  plan[3] = s.plan.chunk_words;
  plan[4] = TU.source;
  plan[5] = (int64_t)TU.table.size();
  plan[6] = s.plan.sync;
  plan[7] = s.plan.wide_levels;
  plan[8] = s.plan.wide_phases;
  int rows = 0;
  for (const auto& r : TU.table) {
    if (!table || rows >= max_rows) break;
    for (int c = 0; c < 7; c++) table[(size_t)rows * 7 + c] = r[c];
    rows++;
  }
  return rows;
}

int gox_topo_info(const gox_topo* t, int64_t* info) {
  if (!t || !info || !t->factored) return GOX_E_INVALID;
  const Schedule& sc = t->sc;
  info[0] = t->jac.n_u;
  info[1] = t->jac.nnz();
  info[2] = (int64_t)t->num.Li.size();
  info[3] = (int64_t)t->num.Ui.size();
  info[4] = sc.n_off;
  info[5] = sc.nblocks;
  info[6] = sc.n_levels;
  info[7] = sc.n_phases;
  info[8] = sc.n_slots;
  info[9] = sc.max_collen;
  const Stream& a = t->s32;
  const Stream& b = t->s64;
  info[10] = a.plan.nw; info[11] = a.plan.ring_rows; info[12] = (int64_t)a.est_cycles;
  info[13] = a.rows_resident; info[14] = a.rows_gathered; info[15] = a.rows_prefetched;
  info[16] = a.rows_late; info[17] = a.rows_jit; info[18] = a.n_steps; info[19] = a.n_waits;
  info[20] = b.plan.nw; info[21] = b.plan.ring_rows; info[22] = (int64_t)b.est_cycles;
  info[23] = b.rows_resident;
  info[24] = a.n_column_cmds;
  info[25] = (int64_t)a.words.size();
  info[28] = a.n_pre;
  info[29] = a.rows_helper;
  info[30] = t->graph_solves;
  info[26] = a.has_bwd ? 1 : 0;
  info[27] = b.has_bwd ? 1 : 0;
  info[31] = a.plan.sync;
  info[32] = a.n_waitp;
  info[33] = a.n_wait_reqs;
  info[34] = a.plan.wide_levels;
  info[35] = a.plan.wide_phases;
  return GOX_OK;
}

int gox_topo_structure(const gox_topo* t, int32_t* Pnum, int32_t* Q, int32_t* R, int32_t* Lp,
                       int32_t* Li, int32_t* Up, int32_t* Ui, double* flops) {
  if (!t || !t->factored) return GOX_E_INVALID;
  const Numeric& N = t->num;
  if (Pnum) std::copy(N.Pnum.begin(), N.Pnum.end(), Pnum);
  if (Q) std::copy(t->sym.Q.begin(), t->sym.Q.end(), Q);
  if (R) std::copy(t->sym.R.begin(), t->sym.R.end(), R);
  if (Lp) std::copy(N.Lp.begin(), N.Lp.end(), Lp);
  if (Li) std::copy(N.Li.begin(), N.Li.end(), Li);
  if (Up) std::copy(N.Up.begin(), N.Up.end(), Up);
  if (Ui) std::copy(N.Ui.begin(), N.Ui.end(), Ui);
  if (flops) { flops[0] = t->sc.flops_refactor; flops[1] = t->sc.flops_solve; }
  return GOX_OK;
}

int gox_topo_jacobian_pattern(const gox_topo* t, int32_t* rows, int32_t* cols) {
  if (!t || !rows || !cols) return GOX_E_INVALID;
  std::copy(t->jac.rows.begin(), t->jac.rows.end(), rows);
  std::copy(t->jac.cols.begin(), t->jac.cols.end(), cols);
  return GOX_OK;
}

int gox_set_timing(gox_topo* t, int32_t enable) {
  if (!t) return GOX_E_INVALID;
  t->timing.on = enable != 0;
  return GOX_OK;
}

int gox_last_timing(const gox_topo* t, double* out) {
  if (!t || !out) return GOX_E_INVALID;
  out[0] = t->timing.iters; out[1] = t->timing.total; out[2] = t->timing.k1;
  out[3] = t->timing.k2; out[4] = t->timing.k3; out[5] = t->timing.k4;
  return GOX_OK;
}

int64_t gox_last_launches(const gox_topo* t) { return t ? t->launches : -1; }

int gox_set_repack(int32_t on) {
  g_repack.store(on ? 1 : 0);
  return GOX_OK;
}

int64_t gox_topo_repacks(const gox_topo* t) {
  if (!t) return -1;
  int64_t r = t->repacks;
  for (const gox_topo* tw = t->twin.get(); tw; tw = tw->twin.get()) r += tw->repacks;
  return r;
}

int gox_set_pivot_tolerance(gox_topo* t, double tol) {
  if (!t || !(tol >= 0.0) || !std::isfinite(tol)) return GOX_E_INVALID;
  t->piv_tol = tol;
  for (gox_topo* tw = t->twin.get(); tw; tw = tw->twin.get()) tw->piv_tol = tol;
  return GOX_OK;
}

int64_t gox_last_fallbacks(const gox_topo* t) { return t ? t->fallbacks : -1; }

int gox_topo_set_zip(gox_topo* t, const double* zi_re, const double* zi_im, const double* zc_re,
                     const double* zc_im) {
  if (!t) return GOX_E_INVALID;
  t->twin.reset();  // rebuilt with the new terms when next needed
  const bool none = !zi_re && !zi_im && !zc_re && !zc_im;
  if (!none && (!zi_re || !zi_im || !zc_re || !zc_im)) return GOX_E_INVALID;
  return guard_impl([&]() -> int {
    const size_t n = (size_t)t->n_bus;
    if (none) {
      t->zip.clear();
      return GOX_OK;
    }
    t->zip.resize(4 * n);
    std::copy(zi_re, zi_re + n, t->zip.begin());
    std::copy(zi_im, zi_im + n, t->zip.begin() + n);
    std::copy(zc_re, zc_re + n, t->zip.begin() + 2 * n);
    std::copy(zc_im, zc_im + n, t->zip.begin() + 3 * n);
    if (int r = require_device()) return r;
    upload(t->dzip, t->zip);
    return GOX_OK;
  });
}

int gox_topo_set_split(gox_topo* t, int32_t parts) {
  if (!t || parts < 0 || parts > 8) return GOX_E_INVALID;
  t->split_parts = parts;
  return GOX_OK;
}

int gox_topo_set_graph(gox_topo* t, int32_t on) {
  if (!t) return GOX_E_INVALID;
  t->graphs_wanted = on != 0;
  for (gox_topo* tw = t->twin.get(); tw; tw = tw->twin.get()) tw->graphs_wanted = on != 0;
  return GOX_OK;
}

int gox_topo_set_initial_guess(gox_topo* t, int32_t mode) {
  if (!t || (mode != GOX_GUESS_GIVEN && mode != GOX_GUESS_LINEAR)) return GOX_E_INVALID;
  t->guess_mode = mode;
  return GOX_OK;
}

int gox_topo_initial_guess(gox_topo* t, int32_t B, const double* p_spec, const double* q_spec,
                           const double* vm0, const double* va0, int32_t v_stride, double* vm_out,
                           double* va_out) {
  if (!t || B <= 0 || !p_spec || !q_spec || !vm0 || !va0 || !vm_out || !va_out) return GOX_E_INVALID;
  if (v_stride != 0 && v_stride != t->n_bus) return GOX_E_INVALID;
  if (int r = require_device()) return r;
  return guard_impl([&]() -> int {
    const int n = t->n_bus;
    const size_t bn = (size_t)B * n, nv = (size_t)(v_stride ? B : 1) * n;
    cudaStream_t st = thread_stream();
    AllocStreamScope alloc_scope(st);
    IoStage& io = t->io;
    io.p.ensure(bn * 8); io.q.ensure(bn * 8); io.vm.ensure(nv * 8); io.va.ensure(nv * 8);
    GOX_CK(cudaMemcpyAsync(io.p.p, p_spec, bn * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(io.q.p, q_spec, bn * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(io.vm.p, vm0, nv * 8, cudaMemcpyHostToDevice, st));
    GOX_CK(cudaMemcpyAsync(io.va.p, va0, nv * 8, cudaMemcpyHostToDevice, st));
    t->guess.d.zip = t->zip.empty() ? nullptr : t->dzip.as<double>();
    if (guess_run(t, B, io.p.as<double>(), io.q.as<double>(), io.vm.as<double>(), io.va.as<double>(),
                  v_stride, nullptr, nullptr, nullptr, st)) {
      GOX_CK(cudaMemcpyAsync(vm_out, t->guess.gvm.p, bn * 8, cudaMemcpyDeviceToHost, st));
      GOX_CK(cudaMemcpyAsync(va_out, t->guess.gva.p, bn * 8, cudaMemcpyDeviceToHost, st));
      GOX_CK(cudaStreamSynchronize(st));
    } else {
      GOX_CK(cudaStreamSynchronize(st));
      for (int s = 0; s < B; s++) {
        std::copy(vm0 + (size_t)s * v_stride, vm0 + (size_t)s * v_stride + n, vm_out + (size_t)s * n);
        std::copy(va0 + (size_t)s * v_stride, va0 + (size_t)s * v_stride + n, va_out + (size_t)s * n);
      }
    }
    return GOX_OK;
  });
}

// ---- LinearSolver level ----------------------------------------------------

int gox_ls_create(int32_t n, int32_t nnz, const int32_t* rows, const int32_t* cols,
                  const double* vals, gox_ls** out) {
  if (!out) return GOX_E_INVALID;
  *out = nullptr;
  if (n <= 0 || nnz < 0 || (nnz > 0 && (!rows || !cols || !vals))) return GOX_E_INVALID;
  for (int e = 0; e < nnz; e++)
    if (rows[e] < 0 || rows[e] >= n || cols[e] < 0 || cols[e] >= n) return GOX_E_INVALID;
  if (int r = require_device()) return r;
  return guard_impl([&]() -> int {
    std::unique_ptr<gox_ls> h(new gox_ls());
    h->n = n;
    h->rows.assign(rows, rows + nnz);
    h->cols.assign(cols, cols + nnz);
    h->csc = build_csc(n, nnz, rows, cols);
    h->sym = klu_analyze(n, h->csc.p.data(), h->csc.i.data());
    h->packed.assign(h->csc.nnz(), 0.0);
    for (int e = 0; e < nnz; e++) h->packed[h->csc.slot_of[e]] += vals[e];
    if (klu_factor(h->csc, h->packed.data(), h->sym, 0.001, h->num) != 0) return GOX_SINGULAR;
    build_schedule(nullptr, h->csc, h->sym, h->num, h->sc);
    make_streams(h->sc, h->s32, h->s64);
    std::vector<int32_t> dummy_p(1, 0), dummy_i;
    std::vector<double> dummy_x;
    h->dsched.load(h->sc, dummy_p, dummy_i, dummy_x, dummy_x);
    h->dsched.load_streams(h->s32, h->s64);
    const SchedDev& S = h->dsched.d;
    h->jbuf.ensure((size_t)S.n_a * 32 * 8 + 8);
    h->lu.ensure((size_t)S.n_slots * 32 * 8 + 8);
    h->off.ensure((size_t)S.n_off * 32 * 8 + 8);
    h->rhs.ensure((size_t)n * 32 * 8);
    h->sol.ensure((size_t)n * 32 * 8);
    h->sing.ensure(128); h->piv.ensure(128); h->gact.ensure(16); h->status.ensure(128);
    int32_t one = 1;
    GOX_CK(cudaMemcpy(h->gact.p, &one, 4, cudaMemcpyHostToDevice));
    *out = h.release();
    return GOX_OK;
  });
}

static int ls_run(gox_ls* h, const double* vals, const double* rhs, double* x) {
  const SchedDev& S = h->dsched.d;
  const int n = h->n;
  // pack duplicates, A order, replicate to all 32 lanes
  std::fill(h->packed.begin(), h->packed.end(), 0.0);
  for (size_t e = 0; e < h->rows.size(); e++) h->packed[h->csc.slot_of[e]] += vals[e];
  // A values in the factor's layout (zeros at fill-in), replicated to 32 lanes
  h->hostbuf.assign((size_t)S.n_slots * 32, 0.0);
  for (int x = 0; x < S.n_slots; x++) {
    const int a = h->sc.slot_a[x];
    if (a >= 0)
      for (int l = 0; l < 32; l++) h->hostbuf[(size_t)x * 32 + l] = h->packed[h->sc.a_csc[a]];
  }
  GOX_CK(cudaMemcpy(h->lu.p, h->hostbuf.data(), h->hostbuf.size() * 8, cudaMemcpyHostToDevice));
  if (h->sc.n_off > 0) {
    std::vector<double> ob((size_t)h->sc.n_off * 32, 0.0);
    for (int x = 0; x < h->sc.n_off; x++)
      for (int l = 0; l < 32; l++) ob[(size_t)x * 32 + l] = h->packed[h->sc.a_csc[h->sc.off_a[x]]];
    GOX_CK(cudaMemcpy(h->off.p, ob.data(), ob.size() * 8, cudaMemcpyHostToDevice));
  }
  std::vector<double> b((size_t)n * 32);
  for (int k = 0; k < n; k++)
    for (int l = 0; l < 32; l++) b[(size_t)k * 32 + l] = rhs[h->num.Pnum[k]];
  GOX_CK(cudaMemcpy(h->rhs.p, b.data(), b.size() * 8, cudaMemcpyHostToDevice));
  GOX_CK(cudaMemset(h->sing.p, 0, 128));
  BatchDev D{};
  D.G = 1;
  D.jbuf = h->jbuf.p; D.lu = h->lu.p; D.off = h->off.p; D.rhs = h->rhs.p; D.sol = h->sol.p;
  D.sing = h->sing.as<int32_t>(); D.piv_flag = h->piv.as<int32_t>(); D.gact = h->gact.as<int32_t>();
  D.piv_tol = 0.0f;
  D.err = h->status.as<int32_t>() + 8;
  GOX_CK(cudaMemset(h->status.p, 0, 128));
  Iter<double>::refactor(h->dsched, D, nullptr);
  Iter<double>::solve_rest(h->dsched, D, nullptr);
  GOX_CK(cudaGetLastError());
  int32_t werr = 0;
  GOX_CK(cudaMemcpy(&werr, h->status.as<int32_t>() + 8, 4, cudaMemcpyDeviceToHost));
  if (werr) return GOX_E_DEVICE_WAIT;
  std::vector<double> X((size_t)n * 32);
  int32_t sing = 0;
  GOX_CK(cudaMemcpy(X.data(), h->sol.p, X.size() * 8, cudaMemcpyDeviceToHost));
  GOX_CK(cudaMemcpy(&sing, h->sing.p, 4, cudaMemcpyDeviceToHost));
  bool finite = true;
  for (int k = 0; k < n; k++) {
    double v = X[(size_t)k * 32];
    x[h->sym.Q[k]] = v;
    if (!std::isfinite(v)) finite = false;
  }
  return (sing || !finite) ? GOX_SINGULAR : GOX_OK;
}

int gox_ls_factor_solve_values(gox_ls* h, const double* vals, const double* rhs, double* x) {
  if (!h || (!vals && !h->rows.empty()) || !rhs || !x) return GOX_E_INVALID;
  return guard_impl([&]() -> int { return ls_run(h, vals, rhs, x); });
}

int gox_ls_factor_solve(gox_ls* h, int32_t nnz, const int32_t* rows, const int32_t* cols,
                        const double* vals, const double* rhs, double* x) {
  if (!h || nnz != (int32_t)h->rows.size()) return h ? GOX_E_PATTERN : GOX_E_INVALID;
  for (int e = 0; e < nnz; e++)
    if (rows[e] != h->rows[e] || cols[e] != h->cols[e]) return GOX_E_PATTERN;
  return gox_ls_factor_solve_values(h, vals, rhs, x);
}

void gox_ls_destroy(gox_ls* h) { delete h; }

}  // extern "C"

// ---- static-scratch LinearSolver variant --------------------------------------
// The scratch of gox_ls_factor_solve_values_static: one fixed device array per
// process (per device), so the call never allocates.  Host code must not take
// its address directly (that is a host-side stand-in); it asks the runtime
// for the device address once per device and passes that to the kernels.
// The address is valid for the device's context; a process that resets the
// device (cudaDeviceReset) must not call this entry afterwards.
namespace gox {
static __device__ __align__(256) unsigned char g_static_scratch[GOX_STATIC_SCRATCH_BYTES];
static void* g_static_addr[256];
static std::mutex g_static_mu;

static int static_scratch(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) {
    cudaGetLastError();
    return GOX_E_CUDA;
  }
  std::lock_guard<std::mutex> lk(g_static_mu);
  if (!g_static_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return GOX_E_CUDA;
    }
    g_static_addr[dev] = p;
  }
  *out = g_static_addr[dev];
  return GOX_OK;
}

// Builds the factor's starting image (A values in the LU layout, zeros at
// fill-in, replicated to the 32 lanes), the permuted right-hand side, and
// clears the flags.
__global__ void k_static_prepare(SchedDev S, const double* packed, const int32_t* acsc,
                                 const double* rhs_raw, const int32_t* pnum, int n, double* lu,
                                 double* off, double* rhsb, int32_t* flags) {
  const size_t total = ((size_t)S.n_slots + (size_t)S.n_off_real + (size_t)n) * 32u;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const size_t e = t >> 5;
    if (e < (size_t)S.n_slots) {
      const int a = S.slot_a[e];
      lu[t] = a >= 0 ? packed[acsc[a]] : 0.0;
    } else if (e < (size_t)S.n_slots + S.n_off_real) {
      const size_t o = e - S.n_slots;
      off[o * 32 + (t & 31)] = packed[acsc[S.off_a[o]]];
    } else {
      const size_t k = e - S.n_slots - S.n_off_real;
      rhsb[k * 32 + (t & 31)] = rhs_raw[pnum[k]];
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < 128) flags[threadIdx.x] = (threadIdx.x == 64) ? 1 : 0;
}

// x[Q[k]] = X[k] (lane 0), flagging non-finite values.
__global__ void k_static_finish(const double* sol, const int32_t* qperm, int n, double* xout,
                                int32_t* flags) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const double v = sol[(size_t)k * 32];
    xout[qperm[k]] = v;
    if (!isfinite(v)) flags[96] = 1;
  }
}
}  // namespace gox

extern "C" int gox_ls_factor_solve_values_static(gox_ls* h, const double* vals,
                                                 const double* rhs, double* x) {
  if (!h || (!vals && !h->rows.empty()) || !rhs || !x) return GOX_E_INVALID;
  return guard_impl([&]() -> int {
    const SchedDev& S = h->dsched.d;
    const int n = h->n;
    // carve the fixed array: 256-byte aligned regions
    size_t off = 0;
    auto take = [&](size_t bytes) {
      size_t o = off;
      off += (bytes + 255) & ~(size_t)255;
      return o;
    };
    const size_t o_lu = take((size_t)S.n_slots * 32 * 8);
    const size_t o_off = take((size_t)std::max(S.n_off_real, 1) * 32 * 8);
    const size_t o_rhs = take((size_t)n * 32 * 8);
    const size_t o_sol = take((size_t)n * 32 * 8);
    const size_t o_pk = take((size_t)h->csc.nnz() * 8);
    const size_t o_acsc = take((size_t)S.n_a * 4);
    const size_t o_rraw = take((size_t)n * 8);
    const size_t o_pnum = take((size_t)n * 4);
    const size_t o_q = take((size_t)n * 4);
    const size_t o_x = take((size_t)n * 8);
    const size_t o_fl = take(128 * 4);
    if (off > (size_t)GOX_STATIC_SCRATCH_BYTES) return GOX_E_TOO_LARGE;
    void* base = nullptr;
    if (int r = static_scratch(&base)) return r;
    unsigned char* B = static_cast<unsigned char*>(base);
    // values of the CSC slots (duplicates summed), as gox_ls_factor_solve_values
    std::fill(h->packed.begin(), h->packed.end(), 0.0);
    for (size_t e = 0; e < h->rows.size(); e++) h->packed[h->csc.slot_of[e]] += vals[e];
    GOX_CK(cudaMemcpy(B + o_pk, h->packed.data(), h->packed.size() * 8, cudaMemcpyHostToDevice));
    GOX_CK(cudaMemcpy(B + o_acsc, h->sc.a_csc.data(), (size_t)S.n_a * 4, cudaMemcpyHostToDevice));
    GOX_CK(cudaMemcpy(B + o_rraw, rhs, (size_t)n * 8, cudaMemcpyHostToDevice));
    GOX_CK(cudaMemcpy(B + o_pnum, h->num.Pnum.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
    GOX_CK(cudaMemcpy(B + o_q, h->sym.Q.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
    int32_t* flags = reinterpret_cast<int32_t*>(B + o_fl);  // [0,32) sing [32,64) piv [64] gact [96] non-finite [100..] wait errors
    const size_t work = ((size_t)S.n_slots + S.n_off_real + n) * 32;
    k_static_prepare<<<grid1d(work), 256>>>(S, reinterpret_cast<double*>(B + o_pk),
                                            reinterpret_cast<int32_t*>(B + o_acsc),
                                            reinterpret_cast<double*>(B + o_rraw),
                                            reinterpret_cast<int32_t*>(B + o_pnum), n,
                                            reinterpret_cast<double*>(B + o_lu),
                                            reinterpret_cast<double*>(B + o_off),
                                            reinterpret_cast<double*>(B + o_rhs), flags);
    BatchDev D{};
    D.G = 1;
    D.lu = B + o_lu; D.off = B + o_off; D.rhs = B + o_rhs; D.sol = B + o_sol;
    D.sing = flags; D.piv_flag = flags + 32; D.gact = flags + 64; D.err = flags + 100;
    D.piv_tol = 0.0f;
    Iter<double>::refactor(h->dsched, D, nullptr);
    Iter<double>::solve_rest(h->dsched, D, nullptr);
    k_static_finish<<<grid1d((size_t)n), 256>>>(reinterpret_cast<double*>(B + o_sol),
                                                reinterpret_cast<int32_t*>(B + o_q), n,
                                                reinterpret_cast<double*>(B + o_x), flags);
    GOX_CK(cudaGetLastError());
    int32_t hf[128];
    GOX_CK(cudaMemcpy(hf, flags, sizeof(hf), cudaMemcpyDeviceToHost));
    GOX_CK(cudaMemcpy(x, B + o_x, (size_t)n * 8, cudaMemcpyDeviceToHost));
    if (hf[100]) return GOX_E_DEVICE_WAIT;
    return (hf[0] || hf[96]) ? GOX_SINGULAR : GOX_OK;
  });
}

// ---- serving -----------------------------------------------------------------
// Worker threads batch queued single-scenario requests per topology
// (continuous batching: while a batch runs, new requests queue; a free
// worker takes the oldest request whose topology has a free lane and up to
// max_batch of that topology's requests in arrival order) and solve each
// batch with gox_batch_solve on the GPU.  A topology's lanes are instances
// of it with their own device state: the topology itself and, once its
// pivot order and plan are fixed, clones of it, so that requests arriving
// while a long batch runs start on another instance instead of waiting for
// it; every instance gives the same result bit for bit.

#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>

namespace gox {
struct ServerReq {
  int64_t ticket = 0;
  int topo = 0;
  std::vector<double> p, q, vm0, va0;
  int32_t slot[4] = {-1, -1, -1, -1};
  double dre[4] = {0, 0, 0, 0}, dim[4] = {0, 0, 0, 0};
  bool outage = false;
  std::chrono::steady_clock::time_point t_submit;
  // results
  int rc = 1;  // 1 pending, 0 done, < 0 error
  std::vector<double> vm, va;
  int32_t iters = 0, status = 0;
  double max_mis = 0, latency = 0;
};
}  // namespace gox

struct gox_server {
  int32_t max_batch = 1024, precision = GOX_PRECISION_MIXED, max_iter = 20;
  double tol = 1e-8;
  int device = 0;
  std::vector<gox_topo*> topos;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::shared_ptr<gox::ServerReq>> queue;
  std::unordered_map<int64_t, std::shared_ptr<gox::ServerReq>> all;
  int64_t next_ticket = 1;
  bool stop = false;
  int64_t batches = 0, solved = 0;
  // HBM budget (0: none): the per-scenario device bytes of each topology's
  // batch buffers bound the batch a worker admits; buffers of idle topologies
  // are released when the reserved total would exceed the budget
  int64_t budget = 0, peak_reserved = 0;
  double queue_s = 0.0, solve_s = 0.0;  // summed over requests: waiting, being solved
  std::vector<int64_t> reserved;  // per topology: its batch and staging buffers
  int64_t reserved_total() const {
    int64_t r = 0;
    for (int64_t v : reserved) r += v;
    return r;
  }
  // Lanes: instance j of topology tp is inst[tp][j] (0: the topology; the
  // others clones made on first use, owned here), busy while a worker
  // solves a batch on it
  static constexpr int kMaxLanes = 8;
  int lanes = 1;
  std::vector<std::array<gox_topo*, kMaxLanes>> inst;
  std::vector<std::array<char, kMaxLanes>> lane_busy;
  std::vector<int> inflight;  // per topology: batches being solved
  // per topology: its pivot order and plan are fixed (recorded by the
  // worker that ran its first batch), so clones of it may be made
  std::vector<char> settled;
  std::vector<std::unique_ptr<gox_topo>> owned;
  int64_t clones = 0;
  // A free lane of topology c (-1: none).  Existing instances first; a new
  // clone only once the topology is settled and without an HBM budget (whose
  // accounting admits one batch per topology).
  int free_lane(int c) const {
    if (!lane_busy[c][0]) return 0;
    const bool grow = budget <= 0 && settled[c];
    for (int j = 1; j < std::min(lanes, kMaxLanes); j++) {
      if (lane_busy[c][j]) continue;
      if (inst[c][j] || grow) return j;
    }
    return -1;
  }
  int64_t held(int tp) const {
    int64_t b = 0;
    for (gox_topo* x : inst[tp])
      if (x) b += held_bytes(x);
    return b;
  }
  // Device bytes a topology's per-batch buffers hold now: its batch and
  // staging buffers, its split twin's, the linear guess system's and the
  // FP64 re-solve staging
  static int64_t held_bytes(gox_topo* t) {
    int64_t b = (int64_t)(t->batch.bytes() + t->io.bytes() + t->pack.bytes() +
                          t->pack_from.bytes);
    for (gox_topo* tw = t->twin.get(); tw; tw = tw->twin.get())
      b += (int64_t)(tw->batch.bytes() + tw->io.bytes());
    for (const gox::DevMem* m : {&t->guess.lu, &t->guess.off, &t->guess.rhs, &t->guess.sol,
                                 &t->guess.sing, &t->guess.piv, &t->guess.gact, &t->guess.err,
                                 &t->guess.gvm, &t->guess.gva, &t->fb.idx, &t->fb.p, &t->fb.q,
                                 &t->fb.vm, &t->fb.va, &t->fb.sl, &t->fb.dr, &t->fb.di, &t->fb.ovm,
                                 &t->fb.ova, &t->fb.it, &t->fb.st, &t->fb.mm, &t->fb.hi})
      b += (int64_t)m->bytes;
    return b;
  }
  static void release_buffers(gox_topo* t) {
    t->batch.release();
    t->io.release();
    t->pack.release();
    t->pack_from.release();
    for (gox_topo* tw = t->twin.get(); tw; tw = tw->twin.get()) {
      tw->batch.release();
      tw->io.release();
    }
    for (gox::DevMem* m : {&t->guess.lu, &t->guess.off, &t->guess.rhs, &t->guess.sol,
                           &t->guess.gvm, &t->guess.gva, &t->fb.idx, &t->fb.p, &t->fb.q, &t->fb.vm,
                           &t->fb.va, &t->fb.sl, &t->fb.dr, &t->fb.di, &t->fb.ovm, &t->fb.ova,
                           &t->fb.it, &t->fb.st, &t->fb.mm, &t->fb.hi})
      m->release();
  }
  // The batch a worker may admit for topology tp under the budget (0: none
  // fits now).  Idle topologies' buffers are released first while one group
  // of 32 scenarios does not fit beside the others'.  Buffers hold whole
  // groups, so the cap is a multiple of 32 (or max_batch); when no other
  // topology holds buffers, one group is admitted even if it exceeds the
  // budget (else the request could never run).
  int admit_cap(int tp) {
    if (budget <= 0) return max_batch;
    const int64_t per = scenario_bytes(topos[tp]);
    auto others = [&]() { return reserved_total() - reserved[tp]; };
    for (size_t o = 0; o < topos.size() && others() + 32 * per > budget; o++)
      if ((int)o != tp && inflight[o] == 0 && reserved[o] > 0) {
        for (gox_topo* x : inst[o])
          if (x) release_buffers(x);
        reserved[o] = 0;
      }
    const int64_t groups = (budget - others()) / (32 * per);
    if (groups <= 0) return others() > 0 ? 0 : std::min(max_batch, 32);
    return (int)std::min<int64_t>(max_batch, groups * 32);
  }
  // Device bytes one scenario of topology t takes in its batch buffers (an
  // upper bound: FP64 width for the typed arrays)
  static int64_t scenario_bytes(const gox_topo* t) {
    const int64_t n = t->n_bus, na = t->jac.nnz(), nu = t->jac.n_u;
    const int64_t slots = t->factored ? (int64_t)t->sc.n_slots + (int64_t)t->sc.n_off : 4 * na;
    return 8 * (8 * n + 5 * n + na + slots + 2 * nu) + 8 * 8 * n + 8 * 64 + 128;
  }
  // Workers: each takes the oldest queued request whose topology has a free
  // lane, with up to max_batch queued requests of that topology, so batches
  // of different topologies, and of one topology on its lanes, run
  // concurrently (each solve has its own stream) while each instance's state
  // is used by one worker at a time.
  static constexpr int kWorkers = 16;
  std::vector<std::thread> workers;

  void run() {
    cudaSetDevice(device);
    for (;;) {
      std::vector<std::shared_ptr<gox::ServerReq>> batch;
      int tp = -1, ln = -1;
      gox_topo* t = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        int cap = 0;
        for (;;) {
          cv.wait(lk, [&] {
            if (stop && queue.empty()) return true;
            for (const auto& r : queue)
              if (free_lane(r->topo) >= 0) return true;
            return false;
          });
          if (stop && queue.empty()) return;
          // topologies in the order of their oldest queued request; the
          // first with a free lane whose batch fits the budget now
          std::vector<char> tried(topos.size(), 0);
          for (const auto& r : queue) {
            const int c = r->topo;
            if (tried[c]) continue;
            tried[c] = 1;
            const int j = free_lane(c);
            if (j < 0) continue;
            cap = admit_cap(c);
            if (cap > 0) {
              tp = c;
              ln = j;
              break;
            }
          }
          if (tp >= 0) break;
          // nothing fits beside the batches being solved: wait for one of
          // them to finish (their buffers then become releasable)
          const int64_t seen = batches;
          cv.wait(lk, [&] { return stop || batches != seen; });
        }
        lane_busy[tp][ln] = 1;
        inflight[tp]++;
        t = inst[tp][ln];
        for (auto it = queue.begin(); it != queue.end() && (int)batch.size() < cap;) {
          if ((*it)->topo == tp) {
            batch.push_back(*it);
            it = queue.erase(it);
          } else {
            ++it;
          }
        }
        // what this batch's buffers will hold (whole groups), counted until
        // its solve reports the real size
        const int64_t groups = ((int64_t)batch.size() + 31) / 32;
        if (budget > 0) reserved[tp] = std::max(reserved[tp], groups * 32 * scenario_bytes(t));
      }
      const auto t_pick = std::chrono::steady_clock::now();
      if (!t) {  // a new lane: clone the topology (outside the lock)
        std::unique_ptr<gox_topo> c;
        try {
          c = clone_factored(topos[tp]);
        } catch (...) {
        }
        std::lock_guard<std::mutex> lk(mu);
        if (c) {
          t = c.get();
          inst[tp][ln] = t;
          owned.push_back(std::move(c));
          clones++;
        } else {  // (no memory for a clone: the batch goes back to the queue)
          for (auto it = batch.rbegin(); it != batch.rend(); ++it) queue.push_front(*it);
          lane_busy[tp][ln] = 0;
          inflight[tp]--;
          lanes = std::max(1, ln);
          cv.notify_all();
          continue;
        }
      }
      solve(t, batch);
      // the topology's refactor plan was timed on its first batch (when the
      // autotuner is on); later batches keep it or a cached plan: no
      // timing inside the serving loop
      t->tune_cache_only = true;
      // (read by the worker that solved on the topology itself: no other
      // thread writes it now)
      const bool fixed = ln == 0 && t->factored && t->guess_mode == 0 && !t->timing.on &&
                         t->tune[precision == GOX_PRECISION_FP64 ? 1 : 0].done;
      const auto t_done = std::chrono::steady_clock::now();
      {
        std::lock_guard<std::mutex> lk(mu);
        if (fixed) settled[tp] = 1;
        for (const auto& r : batch)
          queue_s += std::chrono::duration<double>(t_pick - r->t_submit).count();
        solve_s += std::chrono::duration<double>(t_done - t_pick).count() * (double)batch.size();
        reserved[tp] = held(tp);
        peak_reserved = std::max(peak_reserved, reserved_total());
        lane_busy[tp][ln] = 0;
        inflight[tp]--;
        batches++;
        solved += (int64_t)batch.size();
      }
      cv.notify_all();
    }
  }

  void solve(gox_topo* t, std::vector<std::shared_ptr<gox::ServerReq>>& batch) {
    const int n = t->n_bus, B = (int)batch.size();
    std::vector<double> p((size_t)B * n), q((size_t)B * n), vm0((size_t)B * n), va0((size_t)B * n);
    std::vector<double> vm((size_t)B * n), va((size_t)B * n), mm(B), dre((size_t)B * 4), dim((size_t)B * 4);
    std::vector<int32_t> it(B), st(B), sl((size_t)B * 4, -1);
    bool any_out = false;
    for (int s = 0; s < B; s++) {
      const gox::ServerReq& r = *batch[s];
      std::copy(r.p.begin(), r.p.end(), p.begin() + (size_t)s * n);
      std::copy(r.q.begin(), r.q.end(), q.begin() + (size_t)s * n);
      std::copy(r.vm0.begin(), r.vm0.end(), vm0.begin() + (size_t)s * n);
      std::copy(r.va0.begin(), r.va0.end(), va0.begin() + (size_t)s * n);
      if (r.outage) {
        any_out = true;
        for (int c = 0; c < 4; c++) {
          sl[(size_t)s * 4 + c] = r.slot[c];
          dre[(size_t)s * 4 + c] = r.dre[c];
          dim[(size_t)s * 4 + c] = r.dim[c];
        }
      }
    }
    const int rc = gox_batch_solve(t, B, p.data(), q.data(), vm0.data(), va0.data(), n,
                                   any_out ? sl.data() : nullptr, any_out ? dre.data() : nullptr,
                                   any_out ? dim.data() : nullptr, tol, max_iter, precision,
                                   vm.data(), va.data(), it.data(), st.data(), mm.data(), nullptr);
    const auto now = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(mu);
    for (int s = 0; s < B; s++) {
      gox::ServerReq& r = *batch[s];
      if (rc < 0) {
        r.rc = rc;
      } else {
        r.vm.assign(vm.begin() + (size_t)s * n, vm.begin() + (size_t)(s + 1) * n);
        r.va.assign(va.begin() + (size_t)s * n, va.begin() + (size_t)(s + 1) * n);
        r.iters = it[s];
        r.status = st[s];
        r.max_mis = mm[s];
        r.rc = GOX_OK;
      }
      r.latency = std::chrono::duration<double>(now - r.t_submit).count();
    }
  }
};

extern "C" {

int gox_server_create(int32_t max_batch, int32_t precision, double tol, int32_t max_iter,
                      gox_server** out) {
  if (!out || max_batch <= 0 || max_iter < 0 || !(tol > 0.0) ||
      (precision != GOX_PRECISION_FP64 && precision != GOX_PRECISION_MIXED))
    return GOX_E_INVALID;
  *out = nullptr;
  if (int r = require_device()) return r;
  return guard_impl([&]() -> int {
    std::unique_ptr<gox_server> s(new gox_server());
    s->max_batch = max_batch;
    s->precision = precision;
    s->tol = tol;
    s->max_iter = max_iter;
    GOX_CK(cudaGetDevice(&s->device));
    gox_server* raw = s.get();
    try {
      for (int w = 0; w < gox_server::kWorkers; w++) s->workers.emplace_back([raw] { raw->run(); });
    } catch (...) {
      {
        std::lock_guard<std::mutex> lk(raw->mu);
        raw->stop = true;
      }
      raw->cv.notify_all();
      for (std::thread& w : raw->workers) w.join();
      throw;
    }
    *out = s.release();
    return GOX_OK;
  });
}

int gox_server_add_topology(gox_server* s, gox_topo* t, int32_t* topo_id) {
  if (!s || !t || !topo_id) return GOX_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  s->topos.push_back(t);
  std::array<gox_topo*, gox_server::kMaxLanes> in{};
  in[0] = t;
  s->inst.push_back(in);
  s->lane_busy.push_back({});
  s->inflight.push_back(0);
  s->settled.push_back(0);
  s->reserved.push_back(0);
  *topo_id = (int32_t)s->topos.size() - 1;
  return GOX_OK;
}

int gox_server_submit(gox_server* s, int32_t topo_id, const double* p_spec, const double* q_spec,
                      const double* vm0, const double* va0, const int32_t* out_slot,
                      const double* out_dre, const double* out_dim, int64_t* ticket) {
  if (!s || !p_spec || !q_spec || !vm0 || !va0 || !ticket) return GOX_E_INVALID;
  if ((out_slot != nullptr) != (out_dre != nullptr) || (out_slot != nullptr) != (out_dim != nullptr))
    return GOX_E_INVALID;
  return guard_impl([&]() -> int {
    auto r = std::make_shared<gox::ServerReq>();
    int n = 0;
    {
      // the topology list may grow (and move) under gox_server_add_topology:
      // read the bus count while holding the lock that validates the id
      std::lock_guard<std::mutex> lk(s->mu);
      if (topo_id < 0 || topo_id >= (int32_t)s->topos.size()) return GOX_E_INVALID;
      r->topo = topo_id;
      n = s->topos[topo_id]->n_bus;
    }
    r->p.assign(p_spec, p_spec + n);
    r->q.assign(q_spec, q_spec + n);
    r->vm0.assign(vm0, vm0 + n);
    r->va0.assign(va0, va0 + n);
    if (out_slot) {
      r->outage = true;
      for (int c = 0; c < 4; c++) {
        r->slot[c] = out_slot[c];
        r->dre[c] = out_dre[c];
        r->dim[c] = out_dim[c];
      }
    }
    r->t_submit = std::chrono::steady_clock::now();
    bool budgeted = false;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->stop) return GOX_E_INVALID;
      r->ticket = s->next_ticket++;
      s->all[r->ticket] = r;
      s->queue.push_back(r);
      *ticket = r->ticket;
      budgeted = s->budget > 0;
    }
    // one idle worker takes the request (waking all 16 for every request
    // makes them contend for the lock with the submitting thread); under a
    // budget a worker may be waiting for a batch to finish instead, so all
    if (budgeted) s->cv.notify_all();
    else s->cv.notify_one();
    return GOX_OK;
  });
}

int gox_server_submit_many(gox_server* s, int32_t count, const int32_t* topo_ids,
                           const double* const* p_spec, const double* const* q_spec,
                           const double* const* vm0, const double* const* va0,
                           const int32_t* const* out_slot, const double* const* out_dre,
                           const double* const* out_dim, int64_t* tickets) {
  if (!s || count < 0 || (count > 0 && (!topo_ids || !p_spec || !q_spec || !vm0 || !va0 || !tickets)))
    return GOX_E_INVALID;
  if ((out_slot != nullptr) != (out_dre != nullptr) || (out_slot != nullptr) != (out_dim != nullptr))
    return GOX_E_INVALID;
  if (count == 0) return GOX_OK;
  return guard_impl([&]() -> int {
    std::vector<int> nb(count);
    {
      // every request is checked before any is queued
      std::lock_guard<std::mutex> lk(s->mu);
      for (int k = 0; k < count; k++) {
        const int32_t id = topo_ids[k];
        if (id < 0 || id >= (int32_t)s->topos.size() || !p_spec[k] || !q_spec[k] || !vm0[k] ||
            !va0[k])
          return GOX_E_INVALID;
        if (out_slot && ((out_slot[k] != nullptr) != (out_dre[k] != nullptr) ||
                         (out_slot[k] != nullptr) != (out_dim[k] != nullptr)))
          return GOX_E_INVALID;
        nb[k] = s->topos[id]->n_bus;
      }
    }
    std::vector<std::shared_ptr<gox::ServerReq>> rs(count);
    for (int k = 0; k < count; k++) {
      auto r = std::make_shared<gox::ServerReq>();
      const int n = nb[k];
      r->topo = topo_ids[k];
      r->p.assign(p_spec[k], p_spec[k] + n);
      r->q.assign(q_spec[k], q_spec[k] + n);
      r->vm0.assign(vm0[k], vm0[k] + n);
      r->va0.assign(va0[k], va0[k] + n);
      if (out_slot && out_slot[k]) {
        r->outage = true;
        for (int c = 0; c < 4; c++) {
          r->slot[c] = out_slot[k][c];
          r->dre[c] = out_dre[k][c];
          r->dim[c] = out_dim[k][c];
        }
      }
      rs[k] = std::move(r);
    }
    const auto now = std::chrono::steady_clock::now();
    {
      std::lock_guard<std::mutex> lk(s->mu);
      if (s->stop) return GOX_E_INVALID;
      for (int k = 0; k < count; k++) {
        rs[k]->t_submit = now;
        rs[k]->ticket = s->next_ticket++;
        s->all[rs[k]->ticket] = rs[k];
        s->queue.push_back(rs[k]);
        tickets[k] = rs[k]->ticket;
      }
    }
    if (count == 1 && s->budget <= 0) s->cv.notify_one();
    else s->cv.notify_all();
    return GOX_OK;
  });
}

int gox_server_poll(gox_server* s, int64_t ticket, double* vm, double* va, int32_t* iterations,
                    int32_t* status, double* max_mismatch, double* latency_s) {
  if (!s) return GOX_E_INVALID;
  std::shared_ptr<gox::ServerReq> r;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return GOX_E_INVALID;
    r = it->second;
    if (r->rc == 1) return GOX_PENDING;
    s->all.erase(it);
  }
  if (r->rc < 0) return r->rc;
  if (vm) std::copy(r->vm.begin(), r->vm.end(), vm);
  if (va) std::copy(r->va.begin(), r->va.end(), va);
  if (iterations) *iterations = r->iters;
  if (status) *status = r->status;
  if (max_mismatch) *max_mismatch = r->max_mis;
  if (latency_s) *latency_s = r->latency;
  return GOX_OK;
}

int gox_server_stats(gox_server* s, int64_t* out) {
  if (!s || !out) return GOX_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  out[0] = s->batches;
  out[1] = s->solved;
  out[2] = (int64_t)s->queue.size();
  out[3] = s->reserved_total();
  out[4] = s->peak_reserved;
  out[5] = (int64_t)(s->queue_s * 1e6);
  out[6] = (int64_t)(s->solve_s * 1e6);
  out[7] = s->clones;
  return GOX_OK;
}

int gox_server_set_lanes(gox_server* s, int32_t lanes) {
  if (!s || lanes < 1 || lanes > gox_server::kMaxLanes) return GOX_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  s->lanes = lanes;
  return GOX_OK;
}

int gox_server_set_budget(gox_server* s, int64_t bytes) {
  if (!s || bytes < 0) return GOX_E_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  s->budget = bytes;
  return GOX_OK;
}

void gox_server_destroy(gox_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  for (std::thread& w : s->workers)
    if (w.joinable()) w.join();
  delete s;
}

}  // extern "C"
