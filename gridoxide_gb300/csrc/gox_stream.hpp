// Per-warp command streams for the batched refactor.
//
// The refactor of one topology repeats the same sequence of operations for
// every scenario and every Newton iteration, so all scheduling is done here,
// once per topology, on the host: which warp of the refactor CTA takes which
// column, where in the CTA's shared memory every value lives, which global
// loads are issued a column ahead of their use, and which values are read
// straight from the shared-memory block of the column that produced them
// instead of being loaded again.  The result is, per warp, a list of
// commands that the kernel interprets:
//
//   COLUMN              all of one column (copies for it and for the
//                       warp's next column, wait, steps, FWD, FINISH,
//                       optionally BAR) in one command
//   BWD                 one row of the backward substitution x_k = (y_k -
//                       sum U(k, j) x_j) / U(k, k), with its copies
//   BAR                 __syncthreads (end of a dependency level)
//   GATHER arr m rows   cp.async copies of m rows (one row = one value for
//                       the 32 scenarios of a group) from the factor image,
//                       the forward-substitution vector or the right-hand
//                       side into ring rows; optionally commits the group
//   WAIT n              cp.async.wait_group n, then __syncwarp
//   STEPS m stage       m update steps on the column staged at `stage`
//   FWD                 part of the forward substitution y_k = b_k -
//                       sum L(k, j) y_j (terms in order, in pieces)
//   FINISH              pivot, scale L, write the column back to the factor
//                       and y_k to the forward-substitution vector
//   NEXT                continue with the warp's next stream chunk
//   END
//   PUB n               (plans with progress flags) this warp has finished
//                       its work of the first n dependency levels
//   WAITP               (plans with progress flags) wait until the listed
//                       warps have published the listed level counts
//
// Plans synchronize the levels in one of two ways.  With CTA barriers every
// warp meets every other at the end of every level.  With progress flags
// each warp publishes, per level, that its work of that level
// is done, and before its work of a level waits only for the warps whose
// earlier work it depends on: a value it reads (in a ring or in global
// memory) that they wrote, or a row it overwrites that they read or wrote.
// The compiler finds those dependencies by running the barrier form of the
// same schedule through the host interpreter and recording, for every row,
// its last writer and its readers since (vector clocks keep the waits to
// those not already implied by earlier ones); the flag form then carries
// exactly those waits, and the interpreter checks it again with the flag
// semantics.
//
// Shared memory: per warp two stream chunks (TMA bulk copies) and a ring of
// rows; the rings of all warps form one row space, so a step may read the
// L values of a column finished by any warp while its block is still there.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "gox_engine.hpp"

namespace gox {

enum : int32_t {
  CMD_NOP = 0,
  CMD_BAR = 1,
  CMD_GATHER = 2,
  CMD_WAIT = 3,
  CMD_STEPS = 4,
  CMD_FINISH = 5,
  CMD_NEXT = 6,
  CMD_END = 7,
  CMD_FWD = 8,
  CMD_COLUMN = 9,
  CMD_BWD = 10,
  CMD_PUB = 11,
  CMD_WAITP = 12
};
enum : int32_t { ARR_LU = 0, ARR_X = 1, ARR_RHS = 2 };

constexpr int kStepOps = 9;     // update ops per step (one L(:, j) run piece)
// Rows after the rings of all warps: the zero row (padding terms of the
// forward substitution read it), the trash row (padding copies land in it),
// and rows the unused slots of a step may read.
constexpr int kSpareRows = 12;
constexpr int kMaxRows = 2048;  // ring rows of all warps (11-bit row fields)
constexpr int kMaxRefactorWarps = 12;  // FP32 plans; FP64 plans up to 8 (register budget)

// Encodings (all little fields of 32-bit words):
//   GATHER  w0 = op | m << 4 | commit << 23, then m words src_row | dst_row << 21;
//           source rows number the factor image, then the forward-substitution
//           vector, then the right-hand side as one row space; m is a multiple
//           of the rows one 16-byte per-lane copy moves (4 FP32, 2 FP64),
//           padded with copies of row 0 into the trash row
//   WAIT    w0 = op | n << 4
//   STEPS   w0 = op | m << 4 | stage_row << 16, then (from the next 16-byte
//           boundary) m uint4 steps:
//             x = l_row | j_pos << 16 | cnt << 26    (L values in rows l_row ..,
//                                                     U(j, k) in stage row j_pos)
//             y, z, w = 3 destination stage rows each (10 bits); a step
//             always runs 9 updates, the unused ones on the block's dummy row
//   FWD     w0 = op | m << 4 | first << 20 | real_m << 21, stage_row | len << 16,
//           then m words l_row | y_row << 16 (L(k, j) and y_j): y = (first ? b :
//           y) - sum; m is a multiple of 8, padded with terms on the zero row
//   FINISH  w0 = op, k, base, ulen | llen << 16, stage_row; the stage block
//           is [column rows | y | b | dummy]
//   COLUMN  w0 = op | wait_n << 4 | do_wait << 7 | bar_after << 8 | fwd_continues << 9 |
//           no_finish << 10 (a column's prefix part, or the rest after it), k, base,
//           ulen | llen << 16, stage_row | nlate << 16, npref | nsteps << 16,
//           nfw, real nfw; then nlate gather words (this column, one commit group),
//           npref gather words (the warp's next column, one group), from the
//           next 16-byte boundary nsteps steps, then nfw forward terms: the
//           whole of one column in one command
//   BWD     w0 = op | wait_n << 4 | do_wait << 7 | bar_after << 8 | real_m << 20,
//           k, x_row | y_row << 16, d_row | m << 16, nlate | npref << 16; then
//           the nlate and npref gather words, then m terms u_row | x_row << 16
//           (U(k, j) and x_j; a multiple of 8, padded on the zero row)
//   PUB     w0 = op | n << 4: levels 0 .. n-1 of this warp are done (its
//           writes, and the copies it waited for, are visible to the CTA)
//   WAITP   w0 = op | m << 4, then m words v | n << 8: wait until warp v
//           has published at least n levels (bounded waits)
//   With progress flags, bit 8 of COLUMN / BWD (bar_after) publishes the
//   next level count instead of a barrier.
// Gather word counts are multiples of 2 copies (8 rows FP32, 4 FP64), step
// counts are even, forward term counts multiples of 8 (padding as above);
// 8 words after a command's last step stay inside its chunk (the step loop
// reads the next pair ahead).
struct StreamPlan {
  int elem = 4;             // bytes per value: 4 (FP32) or 8 (FP64)
  int nw = 8;               // warps per CTA
  int ring_rows = 0;        // ring rows per warp
  int big_rows = 0;         // ring rows of warp 0 when larger (columns too
                            // long for the other rings run there); 0: ring_rows
  int chunk_words = 512;    // stream chunk, 32-bit words (multiple of 4)
  int sync = 0;             // levels: 0 CTA barriers, 1 per-warp progress flags
  // The columns of the first wide_levels refactor levels, and their rows of
  // the backward substitution, are not in the stream: the wide kernels run
  // them, one launch per level with one warp per (column or row, group)
  // across all SMs, before the stream kernel (the columns, level by level)
  // and after it (the rows, from the last of those levels down).  Their
  // values reach the stream, and the stream's reach them, through global
  // memory.  wide_phases equals wide_levels (the backward launches).
  int wide_levels = 0, wide_phases = 0;
  int wide_min = 0;   // the narrowest level the split takes (0: no split)
  int wide_rows = 0;  // rows of a wide-kernel warp's stage: the longest wide column
};
// Longest column the wide kernels stage (per warp and lane, in shared memory).
constexpr int kWideCap = 128;
// Narrowest levels the autotuner's wide candidates give the wide kernels:
// the split for batches of many groups, and the deeper one for one or two
// groups of a big grid (the serving shape).
constexpr int kWideMinWidth = 64, kWideMinWidthDeep = 16;
// The wide split of a schedule: the leading refactor levels with at least
// min_width columns each, all columns at most kWideCap long (none when the
// forward substitution is not fused); phases = levels; rows = the longest
// of those columns.
void wide_split(const Schedule& sc, int min_width, int& levels, int& phases, int& rows);
// The rings in the row space: warp 0's first, then the others'.
inline int ring_size(const StreamPlan& p, int w) {
  return w == 0 && p.big_rows > p.ring_rows ? p.big_rows : p.ring_rows;
}
inline int ring_base(const StreamPlan& p, int w) { return w == 0 ? 0 : ring_size(p, 0) + (w - 1) * p.ring_rows; }
inline int ring_total(const StreamPlan& p) { return ring_size(p, 0) + (p.nw - 1) * p.ring_rows; }
inline int ring_warp(const StreamPlan& p, int row) {
  const int r0 = ring_size(p, 0);
  return row < r0 ? 0 : 1 + (row - r0) / p.ring_rows;
}

struct Stream {
  StreamPlan plan;
  std::vector<int32_t> words;            // all chunks; warp w owns chunks chunk0[w] ..
  std::vector<int32_t> chunk0, nchunks;  // per warp
  int n_levels = 0;  // dependency levels in the stream (refactor, then backward substitution)
  int n_bars = 0;    // CTA barriers the stream takes (n_levels, or 0 with progress flags)
  bool has_bwd = false;  // the stream also runs the backward substitution
  // statistics of the schedule
  int64_t rows_gathered = 0, rows_prefetched = 0, rows_resident = 0, rows_late = 0;
  int64_t rows_jit = 0, n_steps = 0, n_waits = 0, n_groups = 0, n_column_cmds = 0, n_pre = 0;
  int64_t rows_helper = 0;  // rows copied by warps idle in the level, for other warps' tasks
  int64_t n_waitp = 0, n_wait_reqs = 0;  // progress-flag waits: commands, warps waited for
  double est_cycles = 0;  // rough critical-path estimate, used to choose a plan
};

// Shared memory (bytes) the refactor kernel needs for a plan.
size_t stream_smem_bytes(const StreamPlan& plan);

// Compiles the refactor of a schedule for a plan (and, with with_bwd, the
// backward substitution after it; the schedule must fuse the forward one).
// Returns false, with the reason, when the plan cannot hold it.
bool build_stream(const Schedule& sc, const StreamPlan& plan, Stream& out, std::string& why,
                  bool with_bwd = false);

// Chooses the plan within `smem_budget` bytes: the most warps (up to 12 in
// FP32, 8 in FP64) whose rings hold the schedule, with the levels' `sync`
// (1 progress flags, 0 barriers), and builds its stream.
// (Measured on GB300, case2000 x 4096 FP32, refactor with both
// substitutions: 8 / 10 / 11 / 12 warps took 2.31 / 2.23 / 2.20 / 2.17 ms
// with 512-, 512-, 256- and 320-word chunks; more warps hide more of the
// latencies of the wide levels and give the narrow ones more idle warps to
// issue copies, and smaller chunks leave the rings room.)
bool choose_stream(const Schedule& sc, int elem, size_t smem_budget, Stream& out,
                   std::string& why, int sync = 0, int wide_min = 0);

// The plans an autotuner may time: warp counts 12, 10, 8, 7, 6, 5 (FP64 up
// to 8) with stream chunks of 320 and 512 words whose rings fit
// `smem_budget`, each without and (when the schedule has one) with the
// wide kernels' split at kWideMinWidth, each with barriers and with
// progress flags, most warps first.
std::vector<StreamPlan> candidate_plans(const Schedule& sc, int elem, size_t smem_budget);

// Builds one plan's stream, with the backward substitution when the
// schedule allows it and the plan holds it, else without.
bool build_plan(const Schedule& sc, const StreamPlan& p, Stream& out, std::string& why);

// Host interpreter of a stream for one scenario in FP64.  lu holds the A
// image in the factor's layout on entry and the factor on exit; X receives
// y_k (forward substitution) when the schedule fuses it.  Checks every
// index, that no row is read before the copy into it is waited for, that
// no copy reads a value before the level that finishes it, and that no two
// warps touch a row within one level when one of them writes it; for a
// plan with progress flags also that every access that conflicts with an
// earlier one of another warp (ring rows, factor values and the solution
// vector in global memory) comes after a wait that orders the two, and
// that every wait is for a level published earlier in level order (so no
// warp can wait forever).  Returns an empty string, or the first violation.
std::string run_stream_host(const Schedule& sc, const Stream& st, std::vector<double>& lu,
                            const std::vector<double>& rhs, std::vector<double>& X,
                            bool& singular);

}  // namespace gox
