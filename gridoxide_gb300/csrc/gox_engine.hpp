// Batched Newton-Raphson engine: per-topology schedule (host) and the device
// state the CUDA kernels run on.
//
// Data layout in HBM ("scenario-interleaved"): scenarios are packed in
// groups of 32 (one warp, one lane per scenario).  Every per-scenario array
// is stored group-major, entry-minor, lane-innermost:
//     value(group g, entry e, lane l) = base[(g * n_entries + e) * 32 + l]
// so one warp access to one entry is one coalesced 128 B (FP32) or 256 B
// (FP64) transaction, and a group's whole factor is one contiguous range.
#pragma once
#include <cstdint>
#include <vector>

#include "gox_symbolic.hpp"

namespace gox {

constexpr int LANES = 32;
constexpr int kMaxBatch = 8;

// Host copy of everything the kernels index; uploaded once per topology
// (after the first numeric factorization fixes the pivot order).
struct Schedule {
  int n_bus = 0, n_u = 0, nnz_y = 0, n_a = 0, n_slots = 0, n_off = 0, nblocks = 0;
  int max_collen = 0, n_levels = 0, n_phases = 0;
  // forward substitution fused into the refactor sweep (only when the BTF
  // form has no off-diagonal entries: the blocks are then independent)
  bool fuse_fwd = false;
  // ---- mismatch / update (per bus)
  std::vector<int32_t> bus_rowP, bus_rowQ;  // bus -> permuted rhs row of its P / Q equation (-1 none)
  std::vector<int32_t> bus_colA, bus_colV;  // bus -> permuted solution index of its angle / |V| unknown
  // ---- Jacobian fill, in refactor consumption order (level by level,
  //      column by column, each column's entries in CSC order)
  std::vector<int32_t> a_kind, a_bi, a_bk, a_yslot;
  // ---- refactor
  std::vector<int32_t> lev_ptr, lev_cols;     // columns grouped by dependency level
  std::vector<int32_t> c_base, c_ulen, c_llen, c_abeg, c_aend;  // per column
  std::vector<int32_t> a_dst;                 // stage position (>=0) or -(off slot + 1)
  std::vector<int32_t> a_csc;                 // CSC slot of A each entry carries
  std::vector<int32_t> op_ptr;                // per column: range into ops (size n+1)
  std::vector<int32_t> op_slot;               // LU slot of the L(i, j) value
  std::vector<uint32_t> op_pos;               // (dst stage pos) | (u stage pos << 16)
  // ops are stored as hazard-free batches (no op of a batch reads or writes
  // a stage entry another op of the batch writes); bt_ptr: per column range
  // into bt_cnt (size n+1), bt_cnt: ops per batch (1..kMaxBatch)
  std::vector<int32_t> bt_ptr;
  std::vector<uint8_t> bt_cnt;
  // per-column packets, 16-byte aligned, in the order the refactor takes
  // columns (lev_cols): everything a warp needs to know about its column,
  // fetched with one bulk copy.  pk_off[q] = int32 offset of the packet of
  // lev_cols[q] (size n+1, last = total):
  //   [0] k  [1] base  [2] ulen  [3] llen  [4] nA  [5] nops  [6] nbt  [7] nfw
  //   [8] jbuf offset of the column's first A entry (entries are contiguous)
  //   [9] first op index  [10..11] unused
  //   nA    stage position of each A entry (>= 0) or -(off slot + 1)
  //   2nfw  (LU slot of L(k, j), j) forward-substitution terms
  //   nbt   batch sizes, 4 per int
  //   2nops (32 * LU slot, 32 * dst | 32 * up << 16) update descriptors,
  //         batch order
  std::vector<int32_t> pk_off, pk;
  // fill recipe in LU layout: per LU slot the A entry it starts from (-1 =
  // fill-in, starts at zero); off-diagonal A entries separately
  std::vector<int32_t> slot_a, off_a;
  // left-looking updates per column, in KLU's order: for column k the U
  // entries p = 0 .. ulen-1 (stage row p holds U(j, k), j = cu_j[cu_ptr[k] + p]);
  // U entry e updates the stage rows cu_dst[cu_dptr[e] ..] with the rows of
  // L(:, j) in stored order.  col_level: dependency level of each column.
  std::vector<int32_t> cu_ptr, cu_j, cu_dptr, cu_dst, col_level;
  int max_pk = 0;    // largest packet, int32 words
  int max_head = 0;  // largest packet without its update descriptors
  int max_ops = 0, max_batches = 0, max_fw = 0;
  // ---- solve (row oriented, KLU block order)
  std::vector<int32_t> ph_ptr, ph_rows, ph_kind;  // phases: rows per phase; kind 0 fwd, 1 bwd
  std::vector<int32_t> fw_ptr, fw_slot, fw_col;   // per row: off (-slot-1) and L(k, j) terms
  std::vector<int32_t> bw_ptr, bw_slot, bw_col;   // per row: U(k, j) terms
  std::vector<int32_t> diag_slot;
  // ---- reference for tests
  double flops_refactor = 0, flops_solve = 0;
};

// Builds the schedule from the first factorization's patterns.
// J may be null (a generic LinearSolver matrix): no fill recipe, no bus maps,
// duplicate triplets allowed.
void build_schedule(const JacPattern* J, const Csc& A, const Symbolic& S, const Numeric& N,
                    Schedule& sc);

// Host FP64 injections and Jacobian fill (used once per topology to obtain
// the Jacobian whose partial-pivoting factorization fixes the pivot order).
void host_injections(int n, const int32_t* yp, const int32_t* yi, const double* yre,
                     const double* yim, const double* vm, const double* va, double* p, double* q);
void host_jac_fill(const JacPattern& J, const double* yre, const double* yim, const double* vm,
                   const double* va, const double* p, const double* q, double* vals);

}  // namespace gox
