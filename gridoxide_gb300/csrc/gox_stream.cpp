// Compiler of the refactor's per-warp command streams, and their host
// interpreter (the CPU check of every stream before it reaches a GPU).
#include "gox_stream.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>
#include <stdexcept>

namespace gox {

size_t stream_smem_bytes(const StreamPlan& p) {
  return (size_t)p.nw * 2 * p.chunk_words * 4 +
         ((size_t)ring_total(p) + kSpareRows) * 32 * p.elem;
}

namespace {

constexpr int64_t kInf = std::numeric_limits<int64_t>::max();
inline int64_t tmake(int level, int64_t pos) { return ((int64_t)level << 32) | pos; }
inline int64_t tend(int level) { return ((int64_t)level << 32) | 0xffffffffLL; }
inline int64_t tagof(int col, int rel) { return ((int64_t)col << 20) | rel; }

// value sources: L runs of an update, forward terms L(k, j) and y_j; for a
// backward-substitution row: y_k, U(k, k), U(k, j) and x_j
enum { IT_LRUN = 0, IT_FWL = 1, IT_FWY = 2, IT_Y = 3, IT_D = 4, IT_U = 5, IT_X = 6 };
enum { TK_COL = 0, TK_BWD = 1 };  // task kinds: a refactor column, a backward row
enum { ST_NONE = 0, ST_GATHERED = 1, ST_RESIDENT = 2 };
constexpr int kPieceRows = 27;  // longest L run piece placed as one block (large rings)

// One value source of a column: a run of rows of another column's result.
struct Item {
  int kind = 0, j = 0;   // producer column
  int src = 0;           // first source row in the row space [factor | X | rhs]
  int rel = 0;           // first row within the producer's stage block
  int nrows = 0;
  int upos = -1;         // L runs: U entry p of the consuming column
  int dfirst = 0;        // L runs: first op of U entry p this piece covers
  int row = -1;          // absolute ring row once placed
  int group = -1;        // commit group of its copy
  int state = ST_NONE;
  bool committed = false;
};

// A task: refactor column k (task k) or backward-substitution row k (task
// n + k, whose block is one row holding x_k).
struct ColInfo {
  int kind = TK_COL;
  int k = 0, level = 0, warp = -1, len = 0, brows = 0, nsteps = 0;
  int block = -1;   // ring row (within its warp's ring) of the stage block
  int group = -1;   // commit group of the stage copy
  bool staged = false, committed = false;
  double cost = 0;
  // A column of a narrow level runs in slices: at each earlier level its
  // warp runs the next updates and forward terms whose sources are finished
  // (in order: a prefix), and the column's own level runs the rest and the
  // finish.  run_early[i] / fw_early[f]: the first level at which run item i
  // / forward pair f (and everything before it) may run.
  int nlr = 0;                   // L-run items (they come first in items)
  std::vector<int> run_early, fw_early;
  int done_runs = 0, done_fw = 0;  // items / forward pairs already run
  bool split = false, fwd_started = false;
  std::vector<Item> items;  // consumption order: L-run pieces (U order), fw pairs
};

struct Emit {
  std::vector<int32_t> w;
  int cw;
  size_t cstart = 0;
  int64_t last_gather = -1;  // word index of the last GATHER header
  explicit Emit(int cw_) : cw(cw_) {}
  size_t room() const { return cstart + cw - 1 - w.size(); }  // last word: NEXT / END
  void next_chunk() {
    w.push_back(CMD_NEXT);
    while (w.size() < cstart + cw) w.push_back(CMD_NOP);
    cstart += cw;
  }
  void need(size_t n) {
    if (room() < n) next_chunk();
  }
};

struct Step {
  uint32_t x, y, z, w;
};

struct Builder {
  const Schedule& sc;
  StreamPlan P;
  int W, R, n;
  int T = 0;  // rows of all rings
  int piece = kPieceRows;  // longest L run piece: shorter with small rings, so two still fit
  int base(int w) const { return ring_base(P, w); }
  int rsize(int w) const { return ring_size(P, w); }
  std::vector<ColInfo> C;
  std::vector<std::vector<int>> seq;
  std::vector<int> seqpos;
  std::vector<int64_t> busy, tag;
  std::vector<int> cursor, ngroups, waited;
  std::vector<int64_t> pos;
  std::vector<Emit> em;
  std::vector<std::vector<Item*>> uncommitted;
  std::vector<std::vector<int>> uncommitted_cols;
  std::vector<std::vector<std::pair<int, int>>> pend_rows;  // copies not yet emitted
  std::vector<int64_t> last_colhdr, last_colend;           // the warp's last COLUMN command
  std::vector<double> wcost;  // per warp, cycles in the current level (estimate)
  std::vector<int> pinned;    // per warp, rows pinned in the current level
  // Copies for the busy warps' next tasks that the level's idle warps issue
  // (one warp issues cp.async copies far slower than the SM takes them from
  // several warps, so the copies of a narrow level's next column go to the
  // warps that would wait at its barrier).  A bundle is one task's copies
  // and the last level whose barrier they must complete before (its
  // deadline): the level before the task's own, or this level when the
  // task is a split column whose slices may start at the next one.  Each
  // helper waits for its share before the deadline's barrier.
  struct Bundle {
    std::vector<std::pair<int, int>> rows;
    int deadline;
  };
  std::vector<Bundle> bundles;
  std::vector<int> idle_warps;
  std::vector<std::vector<std::pair<int, int>>> hpend;  // per warp: helper groups (group, deadline)
  static constexpr int kHelperMinRows = 32;  // same-level helper copies only for prefetches this large
  Stream* out;
  std::string err;

  bool with_bwd = false;  // the backward substitution runs in the stream too
  bool with_pre = true;   // narrow levels' columns run their prefix one level early
  bool with_helpers = true;  // idle warps issue the copies of busy warps' next tasks
  // Plans with progress flags: per warp and level, the WAITP words that open
  // the warp's work of that level (from the analysis of the barrier form).
  const std::vector<std::vector<std::vector<int32_t>>>* reqs = nullptr;
  std::vector<int64_t> last_pub;  // per warp: word index of its last PUB (-1: none to raise)

  Builder(const Schedule& s, const StreamPlan& p) : sc(s), P(p) {
    W = p.nw;
    R = p.ring_rows;
    T = ring_total(p);
    piece = std::max(9, std::min(kPieceRows, R / 6));
    n = s.n_u;
  }

  int64_t now(int w, int L) { return tmake(L, pos[w]++); }

  int alloc(int w, int m, int64_t t) {
    const int Rw = rsize(w);
    if (m > Rw || m <= 0) return -1;
    const int64_t* b = &busy[(size_t)base(w)];
    int run = 0;
    for (int i = 0; i < 2 * Rw; i++) {
      const int r = (cursor[w] + i) % Rw;
      if (r == 0) run = 0;
      if (b[r] < t) {
        if (++run >= m) {
          cursor[w] = (r + 1) % Rw;
          return r - m + 1;
        }
      } else {
        run = 0;
      }
    }
    return -1;
  }
  void take(int w, int r0, int m, int64_t tg_col) {
    for (int i = 0; i < m; i++) {
      busy[(size_t)base(w) + r0 + i] = kInf;
      tag[(size_t)base(w) + r0 + i] = tg_col >= 0 ? tagof((int)tg_col, i) : -1;
    }
  }
  void release_abs(int row, int m, int64_t t) {
    for (int i = 0; i < m; i++) busy[row + i] = t;
  }

  int rpi() const { return 512 / (32 * P.elem); }  // rows per 16-byte-per-lane copy
  // estimated cycles of one warp-wide FMA and of one step: FP64 FMAs run at
  // 1/64 of the FP32 rate on this GPU
  double fma_cost() const { return P.elem == 8 ? 64.0 : 8.0; }
  double step_cost() const { return P.elem == 8 ? 60.0 + 5 * 64.0 : 70.0; }
  int zero_row() const { return T; }
  int trash_row() const { return T + 1; }

  // Source rows of the three arrays as one row space: the factor image,
  // then the forward-substitution vector, then the right-hand side.
  int vrow(int arr, int r) const {
    return arr == ARR_LU ? r : arr == ARR_X ? sc.n_slots + r : sc.n_slots + n + r;
  }
  void emit_gather(int w, int arr, const std::vector<std::pair<int, int>>& rows) {
    for (const auto& r : rows) pend_rows[w].push_back({vrow(arr, r.first), r.second});
  }
  // Pads a copy list to whole pairs of 16-byte-per-lane copies.
  void pad_rows(std::vector<std::pair<int, int>>& rows) const {
    const size_t q = 2 * (size_t)rpi();
    while (rows.size() % q) rows.push_back({0, trash_row()});
  }
  // Gives the copies placed since the last group their commit group (-1 when
  // there are none).
  int new_group(int w) {
    if (uncommitted[w].empty() && uncommitted_cols[w].empty()) return -1;
    const int g = ngroups[w]++;
    out->n_groups++;
    for (Item* it : uncommitted[w]) { it->group = g; it->committed = true; }
    for (int ci : uncommitted_cols[w]) { C[ci].group = g; C[ci].committed = true; }
    uncommitted[w].clear();
    uncommitted_cols[w].clear();
    return g;
  }
  // One GATHER command for every copy issued at this point.
  void flush_gather(int w) {
    std::vector<std::pair<int, int>>& rows = pend_rows[w];
    if (rows.empty()) return;
    Emit& e = em[w];
    const size_t q = 2 * (size_t)rpi();
    pad_rows(rows);
    size_t i = 0;
    while (i < rows.size()) {
      if (e.room() < 1 + q) e.next_chunk();
      size_t m = std::min(rows.size() - i, std::min<size_t>(e.room() - 1, 4092));
      m -= m % q;
      e.last_gather = (int64_t)e.w.size();
      e.w.push_back(CMD_GATHER | (int32_t)(m << 4));
      for (size_t t = 0; t < m; t++) {
        const auto& r = rows[i + t];
        e.w.push_back((int32_t)((uint32_t)r.first | ((uint32_t)r.second << 21)));
      }
      i += m;
    }
    rows.clear();
    pos[w]++;
  }
  void commit(int w) {
    Emit& e = em[w];
    if (uncommitted[w].empty() && uncommitted_cols[w].empty()) return;
    flush_gather(w);
    if (e.last_gather < 0) throw std::logic_error("commit without a gather");
    e.w[e.last_gather] |= (1 << 23);
    new_group(w);
  }
  void wait_for(int w, int g, int L, bool on_path) {
    if (g < 0 || waited[w] >= g) return;
    int m = ngroups[w] - 1 - g;
    if (m < 0) throw std::logic_error("wait for an uncommitted group");
    m = std::min(m, 7);
    Emit& e = em[w];
    e.need(1);
    e.w.push_back(CMD_WAIT | (m << 4));
    waited[w] = ngroups[w] - 1 - m;
    out->n_waits++;
    pos[w]++;
    if (on_path) wcost[w] += 1200;
    (void)L;
  }

  // Places a copy of item `it` (of a column run by warp w) in w's ring.
  bool gather_item(int w, Item& it, int64_t t) {
    const int r = alloc(w, it.nrows, t);
    if (r < 0) return false;
    take(w, r, it.nrows, -1);
    it.row = base(w) + r;
    it.state = ST_GATHERED;
    for (int i = 0; i < it.nrows; i++) pend_rows[w].push_back({it.src + i, it.row + i});
    uncommitted[w].push_back(&it);
    out->rows_gathered += it.nrows;
    return true;
  }

  bool stage_col(int w, int ci, int64_t t) {
    ColInfo& c = C[ci];
    const int r = alloc(w, c.brows, t);
    if (r < 0) return false;
    take(w, r, c.brows, ci);
    c.block = r;
    c.staged = true;
    if (c.kind == TK_BWD) return true;  // x_k is written by the task itself
    std::vector<std::pair<int, int>> rows;
    const int cb = sc.c_base[c.k];
    for (int i = 0; i < c.len; i++) rows.push_back({cb + i, base(w) + r + i});
    emit_gather(w, ARR_LU, rows);
    if (sc.fuse_fwd) emit_gather(w, ARR_RHS, {{c.k, base(w) + r + c.len + 1}});
    uncommitted_cols[w].push_back(ci);
    return true;
  }

  // Reads `it` in place from the producer's block when it is still there,
  // pinning those rows through level L; at most a quarter of a ring is
  // pinned, so the warps keep room for their own copies.
  bool try_resident(Item& it, int L) {
    const ColInfo& pc = C[it.j];
    if (pc.warp < 0 || pc.block < 0 || pc.level >= L) return false;
    const size_t b = (size_t)base(pc.warp) + pc.block + it.rel;
    int fresh = 0;
    for (int i = 0; i < it.nrows; i++) {
      if (tag[b + i] != tagof(it.j, it.rel + i)) return false;
      if (busy[b + i] < tend(L)) fresh++;
    }
    if (pinned[pc.warp] + fresh > rsize(pc.warp) / 4) return false;
    pinned[pc.warp] += fresh;
    it.row = (int)b;
    it.state = ST_RESIDENT;
    for (int i = 0; i < it.nrows; i++) busy[b + i] = std::max(busy[b + i], tend(L));
    out->rows_resident += it.nrows;
    return true;
  }

  // A step that changes nothing the column reads: nine updates of the
  // dummy row (pads step lists to pairs).
  Step dummy_step(const ColInfo& c) const {
    const uint32_t d = (uint32_t)(c.len + 2);
    Step s{};
    s.x = (uint32_t)zero_row();
    s.y = s.z = s.w = d | (d << 10) | (d << 20);
    return s;
  }
  void flush_steps(int w, int stage_abs, std::vector<Step>& steps, const ColInfo& c) {
    Emit& e = em[w];
    if (steps.size() % 2) steps.push_back(dummy_step(c));
    size_t i = 0;
    while (i < steps.size()) {
      // header word, steps (pairs) from the next 4-word boundary, 8 words of
      // over-read room
      const size_t first = (e.w.size() + 1 + 3) & ~(size_t)3;
      if (first + 8 + 8 > e.cstart + e.cw) {
        e.next_chunk();
        continue;
      }
      size_t m = std::min(steps.size() - i, (e.cstart + e.cw - first - 8) / 4);
      m = std::min<size_t>(m, 4094) & ~(size_t)1;
      e.w.push_back(CMD_STEPS | (int32_t)(m << 4) | (stage_abs << 16));
      while (e.w.size() < first) e.w.push_back(0);
      for (size_t q = 0; q < m; q++) {
        const Step& s = steps[i + q];
        e.w.push_back((int32_t)s.x); e.w.push_back((int32_t)s.y);
        e.w.push_back((int32_t)s.z); e.w.push_back((int32_t)s.w);
      }
      i += m;
    }
    steps.clear();
    pos[w]++;
  }

  void add_steps(const ColInfo& c, const Item& it, std::vector<Step>& steps) {
    const int e = sc.cu_ptr[c.k] + it.upos;
    const int d0 = sc.cu_dptr[e] + it.dfirst;
    const uint32_t dummy = (uint32_t)(c.len + 2);
    for (int o = 0; o < it.nrows; o += kStepOps) {
      const int cnt = std::min(kStepOps, it.nrows - o);
      Step s{};
      s.x = (uint32_t)(it.row + o) | ((uint32_t)it.upos << 16) | ((uint32_t)cnt << 26);
      uint32_t d[9];
      for (int t = 0; t < 9; t++) d[t] = dummy;
      for (int t = 0; t < cnt; t++) d[t] = (uint32_t)sc.cu_dst[d0 + o + t];
      s.y = d[0] | (d[1] << 10) | (d[2] << 20);
      s.z = d[3] | (d[4] << 10) | (d[5] << 20);
      s.w = d[6] | (d[7] << 10) | (d[8] << 20);
      steps.push_back(s);
      out->n_steps++;
    }
  }

  // The whole of column c as one COLUMN command, when every value is placed
  // and the command fits in a stream chunk.  g: the last commit group the
  // column's values arrive in.
  // Which part of a column a command runs: L-run items [r0, r1), forward
  // pairs from item f0 to f1, whether the forward sum starts from b, and
  // whether the command finishes the column.
  struct Part {
    size_t r0, r1, f0, f1;
    bool first, finish;
  };
  Part whole(const ColInfo& c) const {
    return {0, (size_t)c.nlr, (size_t)c.nlr, c.items.size(), true, true};
  }
  // the slice of a split column that may run at level L: the next run
  // items and forward pairs whose sources are finished, at most
  // kSliceSteps steps and kSliceTerms terms (a slice runs beside another
  // warp's column; spreading the prefix over the idle levels keeps each
  // level short)
  static constexpr int kSliceSteps = 6, kSliceTerms = 8;
  Part slice_part(const ColInfo& c, int L) const {
    int r1 = c.done_runs, f1 = c.done_fw, steps = 0;
    while (r1 < c.nlr && c.run_early[r1] <= L) {
      const int st = (c.items[r1].nrows + kStepOps - 1) / kStepOps;
      if (steps > 0 && steps + st > kSliceSteps) break;
      steps += st;
      r1++;
    }
    while (f1 < (int)c.fw_early.size() && c.fw_early[f1] <= L && f1 - c.done_fw < kSliceTerms) f1++;
    return {(size_t)c.done_runs, (size_t)r1, (size_t)c.nlr + 2 * (size_t)c.done_fw,
            (size_t)c.nlr + 2 * (size_t)f1, !c.fwd_started, false};
  }
  Part main_part(const ColInfo& c) const {
    return {(size_t)c.done_runs, (size_t)c.nlr, (size_t)c.nlr + 2 * (size_t)c.done_fw, c.items.size(),
            !c.fwd_started, true};
  }
  static bool part_empty(const Part& p) { return p.r0 == p.r1 && p.f0 == p.f1; }

  bool column_cmd(int w, ColInfo& c, int L, std::vector<std::pair<int, int>>& late,
                  std::vector<std::pair<int, int>>& pref, int g, bool on_path, const Part& pt) {
    pad_rows(late);
    pad_rows(pref);
    std::vector<Step> steps;
    const size_t q = pt.r1;
    for (size_t r = pt.r0; r < pt.r1; r++) add_steps(c, c.items[r], steps);
    if (steps.size() % 2) steps.push_back(dummy_step(c));
    std::vector<int32_t> fw;
    size_t nf_real = 0;
    if (sc.fuse_fwd) {
      for (size_t f = pt.f0; f < pt.f1; f += 2)
        fw.push_back(c.items[f].row | (c.items[f + 1].row << 16));
      nf_real = fw.size();
      while (fw.size() % 8) fw.push_back(zero_row() | (zero_row() << 16));
    }
    size_t nl = late.size(), np = pref.size();
    const size_t ns = steps.size(), nf = fw.size();
    auto fits = [&](size_t at, size_t end) {
      const size_t sw = (at + 8 + nl + np + 3) & ~(size_t)3;
      return sw + 4 * ns + nf <= end - 1 && sw + 4 * ns + 8 <= end;
    };
    Emit& e = em[w];
    if ((!fits(0, (size_t)e.cw) || nl > 0xffff || np > 0xffff) && ns <= 0xffff) {
      // the copies as GATHER commands before the command (same commit
      // groups), when the rest fits in a chunk
      nl = np = 0;
      if (fits(0, (size_t)e.cw)) {
        for (auto* rows : {&late, &pref}) {
          if (rows->empty()) continue;
          pend_rows[w].swap(*rows);
          flush_gather(w);
          e.w[e.last_gather] |= (1 << 23);
        }
      } else {
        nl = late.size();
        np = pref.size();
      }
    }
    if (!fits(0, (size_t)e.cw) || nl > 0xffff || np > 0xffff || ns > 0xffff) {
      // the general form counts the steps again
      for (size_t f = pt.r0; f < q; f++)
        out->n_steps -= (c.items[f].nrows + kStepOps - 1) / kStepOps;
      return false;
    }
    if (!fits(e.w.size(), e.cstart + e.cw)) e.next_chunk();
    int32_t w0 = CMD_COLUMN | (pt.first ? 0 : (1 << 9)) | (pt.finish ? 0 : (1 << 10));
    if (g >= 0 && waited[w] < g) {
      const int m = std::min(ngroups[w] - 1 - g, 7);
      w0 |= (m << 4) | (1 << 7);
      waited[w] = ngroups[w] - 1 - m;
      out->n_waits++;
      if (on_path) wcost[w] += 1200;
    }
    const int stage_abs = base(w) + c.block;
    last_colhdr[w] = (int64_t)e.w.size();
    e.w.push_back(w0);
    e.w.push_back(c.k);
    e.w.push_back(sc.c_base[c.k]);
    e.w.push_back(sc.c_ulen[c.k] | (sc.c_llen[c.k] << 16));
    e.w.push_back(stage_abs | (int32_t)(nl << 16));
    e.w.push_back((int32_t)(np | (ns << 16)));
    e.w.push_back((int32_t)nf);
    e.w.push_back((int32_t)nf_real);
    for (const auto& r : late) e.w.push_back((int32_t)((uint32_t)r.first | ((uint32_t)r.second << 21)));
    for (const auto& r : pref) e.w.push_back((int32_t)((uint32_t)r.first | ((uint32_t)r.second << 21)));
    while (e.w.size() % 4) e.w.push_back(0);
    for (const Step& st : steps) {
      e.w.push_back((int32_t)st.x); e.w.push_back((int32_t)st.y);
      e.w.push_back((int32_t)st.z); e.w.push_back((int32_t)st.w);
    }
    for (int32_t x : fw) e.w.push_back(x);
    last_colend[w] = (int64_t)e.w.size();
    out->n_column_cmds++;
    pos[w]++;
    const int64_t tf = now(w, L);
    for (size_t r = pt.r0; r < pt.r1; r++)
      if (c.items[r].state == ST_GATHERED) release_abs(c.items[r].row, c.items[r].nrows, tf);
    for (size_t f = pt.f0; f < pt.f1; f++)
      if (c.items[f].state == ST_GATHERED) release_abs(c.items[f].row, c.items[f].nrows, tf);
    if (pt.finish) release_abs(stage_abs, c.brows, tf);
    wcost[w] += step_cost() * ns + 80 + (pt.finish ? (4.0 + fma_cost()) * c.len : 0.0) +
                fma_cost() * nf_real;
    return true;
  }

  // A slice of split column ci on its warp w during level L (before the
  // column's own level): its stage (first slice), the copies of the slice's
  // values, its steps and forward terms, as one COLUMN command without
  // finish.  When something does not fit, the copies placed so far stay for
  // the column, values read in place are decided again, and the rest of the
  // column runs at its own level.
  void run_slice(int w, int ci, int L) {
    ColInfo& c = C[ci];
    const Part pt = slice_part(c, L);
    if (part_empty(pt)) return;
    auto undo_in_place = [&]() {
      for (size_t r = pt.r0; r < pt.r1; r++)
        if (c.items[r].state == ST_RESIDENT) { c.items[r].state = ST_NONE; c.items[r].row = -1; }
      for (size_t f = pt.f0; f < pt.f1; f++)
        if (c.items[f].state == ST_RESIDENT) { c.items[f].state = ST_NONE; c.items[f].row = -1; }
    };
    const int64_t t = now(w, L);
    bool waited_late = false;
    if (!c.staged) {
      if (!stage_col(w, ci, t)) {
        c.split = false;
        undo_in_place();
        return;
      }
      waited_late = true;
    }
    bool ok = true;
    auto place = [&](Item& it) {
      if (it.state == ST_NONE) {
        if (gather_item(w, it, t)) { out->rows_late += it.nrows; waited_late = true; }
        else ok = false;
      }
    };
    for (size_t r = pt.r0; r < pt.r1 && ok; r++) place(c.items[r]);
    for (size_t f = pt.f0; f < pt.f1 && ok; f++) place(c.items[f]);
    std::vector<std::pair<int, int>> late_rows, none;
    late_rows.swap(pend_rows[w]);
    new_group(w);
    int g = c.group;
    for (size_t r = pt.r0; r < pt.r1; r++)
      if (c.items[r].state == ST_GATHERED) g = std::max(g, c.items[r].group);
    for (size_t f = pt.f0; f < pt.f1; f++)
      if (c.items[f].state == ST_GATHERED) g = std::max(g, c.items[f].group);
    if (ok && column_cmd(w, c, L, late_rows, none, g, waited_late, pt)) {
      c.done_runs = (int)pt.r1;
      c.done_fw = (int)(pt.f1 - (size_t)c.nlr) / 2;
      c.fwd_started = true;
      out->n_pre++;
      return;
    }
    c.split = false;
    undo_in_place();
    if (!late_rows.empty()) {
      pend_rows[w].swap(late_rows);
      flush_gather(w);
      em[w].w[em[w].last_gather] |= (1 << 23);
    }
  }

  // Issues the block of the warp's next task and every value of it finished
  // before level L ahead of time: by this warp (one commit group, in the
  // command's prefetch list, waited for when that task starts), or, when
  // the level has idle warps and the task runs at a later level, by the
  // idle warps (see Bundle), as are then the values of the tasks after it
  // whose deadline is after this level (up to kHelperAhead tasks ahead).
  // Copies by idle warps run concurrently with this warp's tasks, so their
  // rows must be free during the whole level.
  static constexpr int kHelperAhead = 1;
  void prefetch_next(int w, int ci, int L, int64_t t, std::vector<std::pair<int, int>>& pref_rows) {
    const int sp = seqpos[ci];
    const int nseq = (int)seq[w].size();
    const bool can_help = !idle_warps.empty() && sp + 1 < nseq && C[seq[w][sp + 1]].level > L;
    // the last level whose barrier the copies for task d must complete
    // before: the one before the task's own, or, for a split column whose
    // slices may start once the warp's previous task is done, that task's
    auto deadline_of = [&](int d) {
      const ColInfo& nc = C[seq[w][sp + d]];
      const int prev = d == 1 ? L : C[seq[w][sp + d - 1]].level;
      return (nc.kind == TK_COL && nc.split) ? prev : nc.level - 1;
    };
    auto rows_needed = [&](const ColInfo& nc) {
      int rows = nc.staged || nc.kind == TK_BWD ? 0 : nc.len + (sc.fuse_fwd ? 1 : 0);
      for (const Item& it : nc.items)
        if (it.state == ST_NONE && C[it.j].level < L) rows += it.nrows;
      return rows;
    };
    auto place = [&](int d, int64_t tt) -> bool {
      const int ni = seq[w][sp + d];
      ColInfo& nc = C[ni];
      if (!nc.staged && !stage_col(w, ni, tt)) return false;
      for (Item& it : nc.items) {
        if (it.state != ST_NONE || C[it.j].level >= L) continue;
        if (!gather_item(w, it, tt)) return false;
        out->rows_prefetched += it.nrows;
      }
      return true;
    };
    auto to_helpers = [&](int deadline) {
      // complete before the deadline's barrier: nothing for this warp to wait for
      for (Item* it : uncommitted[w]) { it->group = -1; it->committed = true; }
      for (int c2 : uncommitted_cols[w]) { C[c2].group = -1; C[c2].committed = true; }
      uncommitted[w].clear();
      uncommitted_cols[w].clear();
      out->rows_helper += (int64_t)pend_rows[w].size();
      if (!pend_rows[w].empty()) bundles.push_back({std::move(pend_rows[w]), deadline});
      pend_rows[w].clear();
    };
    if (sp + 1 >= nseq) return;
    const int d1 = can_help ? deadline_of(1) : L;
    const int need1 = rows_needed(C[seq[w][sp + 1]]);
    const bool h1 = can_help && need1 > 0 && (d1 > L || need1 >= kHelperMinRows);
    const bool ok = place(1, h1 ? tmake(L, 0) : t);
    if (h1) {
      to_helpers(d1);
    } else {
      pref_rows.swap(pend_rows[w]);
      new_group(w);
    }
    if (!ok || !can_help) return;
    for (int d = 2; d <= kHelperAhead && sp + d < nseq; d++) {
      const int dd = deadline_of(d);
      if (dd <= L) break;
      const bool okd = place(d, tmake(L, 0));
      to_helpers(dd);
      if (!okd) break;
    }
  }

  // The idle warp h issues its share of the level's helper copies (one
  // commit group) before its own slice; helper_wait then waits for them
  // before the level's barrier.
  void helper_gather(int h, std::vector<std::pair<int, int>>& rows, int deadline) {
    if (rows.empty()) return;
    if (!pend_rows[h].empty()) throw std::logic_error("helper copies with copies pending");
    const size_t nreal = rows.size();
    pend_rows[h].swap(rows);
    flush_gather(h);
    em[h].w[em[h].last_gather] |= (1 << 23);
    const int g = ngroups[h]++;
    out->n_groups++;
    wcost[h] += 70.0 * (double)((nreal + rpi() - 1) / rpi());
    hpend[h].push_back({g, deadline});
  }
  // Before warp h's barrier of level L: waits for its helper groups due.
  void helper_wait(int h, int L) {
    int g = -1;
    for (const auto& pg : hpend[h])
      if (pg.second <= L) g = std::max(g, pg.first);
    if (g < 0) return;
    wait_for(h, g, L, false);
    std::vector<std::pair<int, int>> keep;
    for (const auto& pg : hpend[h])
      if (pg.first > g) keep.push_back(pg);
    hpend[h].swap(keep);
    wcost[h] += 1000;
  }

  // The index in seq[w] of the warp's next task after its level-L tasks
  // (from q0), when that is a split column of a later level; else -1.
  int next_own(int w, int q0, int L) const {
    int q = q0;
    while (q < (int)seq[w].size() && C[seq[w][q]].level <= L) q++;
    if (q >= (int)seq[w].size()) return -1;
    const ColInfo& c = C[seq[w][q]];
    return (c.kind == TK_COL && c.split && c.level > L) ? q : -1;
  }

  // x_k = (y_k - sum U(k, j) x_j) / U(k, k) as one BWD command.
  bool run_bwd(int w, int ci, int L) {
    ColInfo& c = C[ci];
    int64_t t = now(w, L);
    bool waited_late = false;
    if (!c.staged && !stage_col(w, ci, t)) {
      err = "no ring room for the row of backward task " + std::to_string(c.k);
      return false;
    }
    for (Item& it : c.items)
      if (it.state == ST_NONE && gather_item(w, it, t)) {
        out->rows_late += it.nrows;
        waited_late = true;
      }
    std::vector<std::pair<int, int>> late_rows, pref_rows;
    late_rows.swap(pend_rows[w]);
    new_group(w);
    bool placed = true;
    for (const Item& it : c.items) placed = placed && it.state != ST_NONE;
    if (placed) prefetch_next(w, ci, L, t, pref_rows);
    int g = c.group;
    for (const Item& it : c.items)
      if (it.state == ST_GATHERED) g = std::max(g, it.group);
    pad_rows(late_rows);
    pad_rows(pref_rows);
    const size_t nterm = (c.items.size() - 2) / 2;
    const size_t mpad = (nterm + 7) & ~(size_t)7;
    Emit& e = em[w];
    if (!placed || 5 + late_rows.size() + pref_rows.size() + mpad > (size_t)e.cw - 1) {
      // general form: copies as single commands, the rest just in time
      for (auto* rows : {&late_rows, &pref_rows}) {
        if (rows->empty()) continue;
        pend_rows[w].swap(*rows);
        flush_gather(w);
        e.w[e.last_gather] |= (1 << 23);
      }
      wait_for(w, g, L, waited_late);
      if (!placed) {
        const int64_t tj = now(w, L);
        for (Item& it : c.items)
          if (it.state == ST_NONE) {
            if (!gather_item(w, it, tj)) {
              err = "no ring room for backward task " + std::to_string(c.k);
              return false;
            }
            out->rows_jit += it.nrows;
          }
        commit(w);
        int gg = -1;
        for (const Item& it : c.items)
          if (it.state == ST_GATHERED) gg = std::max(gg, it.group);
        wait_for(w, gg, L, true);
      }
      late_rows.clear();
      pref_rows.clear();
      g = -1;
      if (5 + mpad > (size_t)e.cw - 1) {
        err = "backward row too long for a stream chunk";
        return false;
      }
    }
    const size_t need = 5 + late_rows.size() + pref_rows.size() + mpad;
    e.need(need);
    int32_t w0 = CMD_BWD | (int32_t)(nterm << 20);
    if (g >= 0 && waited[w] < g) {
      const int m = std::min(ngroups[w] - 1 - g, 7);
      w0 |= (m << 4) | (1 << 7);
      waited[w] = ngroups[w] - 1 - m;
      out->n_waits++;
      if (waited_late) wcost[w] += 1200;
    }
    const int xrow = base(w) + c.block;
    last_colhdr[w] = (int64_t)e.w.size();
    e.w.push_back(w0);
    e.w.push_back(c.k);
    e.w.push_back(xrow | (c.items[0].row << 16));
    e.w.push_back(c.items[1].row | (int32_t)(mpad << 16));
    e.w.push_back((int32_t)(late_rows.size() | (pref_rows.size() << 16)));
    for (const auto& r : late_rows) e.w.push_back((int32_t)((uint32_t)r.first | ((uint32_t)r.second << 21)));
    for (const auto& r : pref_rows) e.w.push_back((int32_t)((uint32_t)r.first | ((uint32_t)r.second << 21)));
    for (size_t q = 0; q < nterm; q++)
      e.w.push_back(c.items[2 + 2 * q].row | (c.items[3 + 2 * q].row << 16));
    for (size_t q = nterm; q < mpad; q++) e.w.push_back(zero_row() | (zero_row() << 16));
    last_colend[w] = (int64_t)e.w.size();
    pos[w]++;
    const int64_t tf = now(w, L);
    for (const Item& it : c.items)
      if (it.state == ST_GATHERED) release_abs(it.row, it.nrows, tf);
    release_abs(xrow, c.brows, tf);
    wcost[w] += 100 + fma_cost() * (double)nterm;
    return true;
  }

  // Emits everything of column ci (warp w, level L).
  bool run_col(int w, int ci, int L) {
    ColInfo& c = C[ci];
    if (c.kind == TK_BWD) return run_bwd(w, ci, L);
    int64_t t = now(w, L);
    bool waited_late = false;
    if (!c.staged) {
      if (!stage_col(w, ci, t)) {
        err = "no ring room for the stage block of column " + std::to_string(c.k);
        return false;
      }
      waited_late = true;  // the stage copy was not issued ahead
    }
    for (Item& it : c.items)
      if (it.state == ST_NONE && gather_item(w, it, t)) {
        out->rows_late += it.nrows;
        waited_late = true;
      }
    std::vector<std::pair<int, int>> late_rows, pref_rows;
    late_rows.swap(pend_rows[w]);
    new_group(w);
    // the warp's next column: its stage block and every value finished before
    // this level, issued now and waited for when that column starts
    // (only when this column has every value placed: a prefetch must not
    // take the room this column still needs)
    bool placed = true;
    for (const Item& it : c.items) placed = placed && it.state != ST_NONE;
    if (placed) prefetch_next(w, ci, L, t, pref_rows);
    int g = c.group;
    for (const Item& it : c.items)
      if (it.state == ST_GATHERED) g = std::max(g, it.group);
    const Part mp = main_part(c);
    if (placed && column_cmd(w, c, L, late_rows, pref_rows, g, waited_late, mp)) return true;
    // the general form: single commands, values fetched in pieces as room allows
    for (auto* rows : {&late_rows, &pref_rows}) {
      if (rows->empty()) continue;
      pend_rows[w].swap(*rows);
      flush_gather(w);
      em[w].w[em[w].last_gather] |= (1 << 23);
    }
    wait_for(w, g, L, waited_late);
    // updates, fetching values that found no room just in time
    std::vector<Step> steps;
    std::vector<Item*> consumed;
    const int stage_abs = base(w) + c.block;
    auto release_consumed = [&]() {
      const int64_t tf = now(w, L);
      for (Item* it : consumed) release_abs(it->row, it->nrows, tf);
      consumed.clear();
    };
    auto jit = [&](size_t from) -> bool {
      flush_steps(w, stage_abs, steps, c);
      release_consumed();
      const int64_t tj = now(w, L);
      bool any = false;
      for (size_t q = from; q < c.items.size(); q++) {
        Item& it = c.items[q];
        if (it.state != ST_NONE) continue;
        if (!gather_item(w, it, tj)) break;
        out->rows_jit += it.nrows;
        any = true;
      }
      if (!any) return false;
      commit(w);
      int gg = -1;
      for (size_t q = from; q < c.items.size(); q++)
        if (c.items[q].state == ST_GATHERED) gg = std::max(gg, c.items[q].group);
      wait_for(w, gg, L, true);
      return true;
    };
    size_t q = mp.r0;
    for (; q < mp.r1; q++) {
      Item& it = c.items[q];
      if (it.state == ST_NONE && !jit(q)) {
        err = "no ring room for an update run of column " + std::to_string(c.k);
        return false;
      }
      add_steps(c, it, steps);
      wcost[w] += step_cost() * ((it.nrows + kStepOps - 1) / kStepOps);
      if (it.state == ST_GATHERED) consumed.push_back(&it);
    }
    flush_steps(w, stage_abs, steps, c);
    release_consumed();
    // forward substitution y_k = b_k - sum L(k, j) y_j, in order, in pieces
    // whose values fit in the ring
    Emit& e = em[w];
    q = mp.f0;
    if (sc.fuse_fwd) {
      size_t f = q;
      bool first = mp.first;
      do {
        if (f < c.items.size()) {
          const size_t h = c.items[f].state == ST_NONE ? f : f + 1;
          if (c.items[h].state == ST_NONE && !jit(h)) {
            err = "no ring room for the forward terms of column " + std::to_string(c.k);
            return false;
          }
        }
        size_t f1 = f;
        while (f1 < c.items.size() && c.items[f1].state != ST_NONE && c.items[f1 + 1].state != ST_NONE)
          f1 += 2;
        size_t a0 = f;
        do {  // FWD commands over pairs a0 .. f1 (split at chunk ends)
          e.need(2 + 8);
          size_t m = std::min((f1 - a0) / 2, (e.room() - 2) & ~(size_t)7);
          const size_t mp = (m + 7) & ~(size_t)7;
          e.w.push_back(CMD_FWD | (int32_t)(mp << 4) | (first ? (1 << 20) : 0) | (int32_t)(m << 21));
          e.w.push_back(stage_abs | (c.len << 16));
          for (size_t t = 0; t < m; t++) {
            const Item& la = c.items[a0 + 2 * t];
            const Item& ya = c.items[a0 + 2 * t + 1];
            e.w.push_back(la.row | (ya.row << 16));
          }
          for (size_t t = m; t < mp; t++) e.w.push_back(zero_row() | (zero_row() << 16));
          first = false;
          a0 += 2 * m;
        } while (a0 < f1);
        pos[w]++;
        const int64_t tr = now(w, L);
        for (size_t t = f; t < f1; t++)
          if (c.items[t].state == ST_GATHERED) release_abs(c.items[t].row, c.items[t].nrows, tr);
        f = f1;
      } while (f < c.items.size());
    }
    // finish
    e.need(5);
    e.w.push_back(CMD_FINISH);
    e.w.push_back(c.k);
    e.w.push_back(sc.c_base[c.k]);
    e.w.push_back(sc.c_ulen[c.k] | (sc.c_llen[c.k] << 16));
    e.w.push_back(stage_abs);
    const int nfw = (int)(c.items.size() - q) / 2;
    const int64_t tf = now(w, L);
    release_abs(stage_abs, c.brows, tf);
    wcost[w] += 80 + (4.0 + fma_cost()) * c.len + fma_cost() * nfw;
    return true;
  }

  bool build(Stream& st) {
    out = &st;
    st = Stream();
    st.plan = P;
    if (R <= 0 || W <= 0 || P.chunk_words % 4 || P.chunk_words < 64) {
      err = "bad plan";
      return false;
    }
    if (T + kSpareRows > kMaxRows) {
      err = "ring rows exceed the 11-bit row fields";
      return false;
    }
    if (sc.n_slots >= (1 << 21) || n >= (1 << 21)) {
      err = "factor too large for 21-bit row fields";
      return false;
    }
    // levels the wide kernels run before the stream (their columns are
    // finished in global memory when it starts: level -1 here) and backward
    // phases they run after it
    const int S0 = P.wide_levels, PW = P.wide_phases;
    if (S0 < 0 || S0 >= sc.n_levels || PW != S0 || (S0 > 0 && !(sc.fuse_fwd && with_bwd)) ||
        (S0 > 0 && (P.wide_rows <= 0 || P.wide_rows > kWideCap))) {
      err = "bad wide split";
      return false;
    }
    const int NR = sc.n_levels - S0;  // refactor levels in the stream
    // ---- columns and their value sources
    C.assign(n, ColInfo());
    for (int k = 0; k < n; k++) {
      ColInfo& c = C[k];
      c.k = k;
      c.level = sc.col_level[k] < S0 ? -1 : sc.col_level[k] - S0;
      c.len = sc.c_ulen[k] + 1 + sc.c_llen[k];
      c.brows = c.len + 3;
      if (c.level >= 0 && c.len >= 1024) {
        err = "column too long for 10-bit stage rows";
        return false;
      }
      if (c.level >= 0 && c.brows > rsize(0)) {
        err = "column " + std::to_string(k) + " longer than the ring";
        return false;
      }
      for (int p = 0; p < sc.c_ulen[k]; p++) {
        const int e = sc.cu_ptr[k] + p;
        const int j = sc.cu_j[e];
        const int nl = sc.c_llen[j];
        for (int d = 0; d < nl; d += piece) {
          Item it;
          it.kind = IT_LRUN;
          it.j = j;
          it.rel = sc.c_ulen[j] + 1 + d;
          it.src = sc.c_base[j] + it.rel;
          it.nrows = std::min(piece, nl - d);
          it.upos = p;
          it.dfirst = d;
          c.items.push_back(it);
          c.nsteps += (it.nrows + kStepOps - 1) / kStepOps;
        }
      }
      c.nlr = (int)c.items.size();
      if (sc.fuse_fwd) {
        for (int tt = sc.fw_ptr[k]; tt < sc.fw_ptr[k + 1]; tt++) {
          const int slot = sc.fw_slot[tt], j = sc.fw_col[tt];
          if (slot < 0) {
            err = "fused forward substitution with off-diagonal terms";
            return false;
          }
          Item a;
          a.kind = IT_FWL;
          a.j = j;
          a.src = slot;
          a.rel = slot - sc.c_base[j];
          a.nrows = 1;
          Item b;
          b.kind = IT_FWY;
          b.j = j;
          b.src = sc.n_slots + j;
          b.rel = sc.c_ulen[j] + 1 + sc.c_llen[j];
          b.nrows = 1;
          c.items.push_back(a);
          c.items.push_back(b);
        }
      }
      c.cost = 40 + step_cost() * c.nsteps + 4.0 * c.len +
               fma_cost() * (sc.fuse_fwd ? sc.fw_ptr[k + 1] - sc.fw_ptr[k] : 0);
    }
    // ---- backward-substitution rows (tasks n + k), after the refactor's
    //      levels: x_k = (y_k - sum U(k, j) x_j) / U(k, k)
    int n_blev = 0;
    std::vector<int32_t> blev_ptr(1, 0), blev_rows;
    if (with_bwd) {
      C.resize(2 * (size_t)n);
      // phases as scheduled, without the rows of the wide kernels' columns
      // (solved after the stream, in reverse level order; no row of the
      // stream needs them: a row needs rows of higher refactor levels only)
      for (int ph = 0; ph < sc.n_phases; ph++) {
        if (sc.ph_kind[ph] != 1) {
          err = "backward tasks need a schedule without forward phases";
          return false;
        }
        const size_t before = blev_rows.size();
        for (int q = sc.ph_ptr[ph]; q < sc.ph_ptr[ph + 1]; q++) {
          const int k = sc.ph_rows[q];
          if (sc.col_level[k] < S0) continue;
          ColInfo& c = C[n + k];
          c.kind = TK_BWD;
          c.k = k;
          c.level = NR + n_blev;
          c.brows = 1;
          const int ulen = sc.c_ulen[k], len = ulen + 1 + sc.c_llen[k];
          Item y;
          y.kind = IT_Y; y.j = k; y.src = sc.n_slots + k; y.rel = len; y.nrows = 1;
          Item d;
          d.kind = IT_D; d.j = k; d.src = sc.c_base[k] + ulen; d.rel = ulen; d.nrows = 1;
          c.items.push_back(y);
          c.items.push_back(d);
          for (int tt = sc.bw_ptr[k]; tt < sc.bw_ptr[k + 1]; tt++) {
            const int slot = sc.bw_slot[tt], j = sc.bw_col[tt];
            Item u;
            u.kind = IT_U; u.j = j; u.src = slot; u.rel = slot - sc.c_base[j]; u.nrows = 1;
            Item xj;
            xj.kind = IT_X; xj.j = n + j; xj.src = sc.n_slots + j; xj.rel = 0; xj.nrows = 1;
            c.items.push_back(u);
            c.items.push_back(xj);
          }
          c.cost = 100 + fma_cost() * (sc.bw_ptr[k + 1] - sc.bw_ptr[k]);
          blev_rows.push_back(n + k);
        }
        if (blev_rows.size() == before) continue;  // every row of the phase is a wide one
        blev_ptr.push_back((int32_t)blev_rows.size());
        n_blev++;
      }
    }
    const int NL = NR + n_blev;
    if (NL <= 0) {
      err = "no level left for the stream";
      return false;
    }
    auto level_tasks = [&](int L) {
      if (L < NR)
        return std::vector<int>(sc.lev_cols.begin() + sc.lev_ptr[L + S0],
                                sc.lev_cols.begin() + sc.lev_ptr[L + S0 + 1]);
      const int b = L - NR;
      return std::vector<int>(blev_rows.begin() + blev_ptr[b], blev_rows.begin() + blev_ptr[b + 1]);
    };
    // ---- columns to warps: per level, longest first to the least loaded
    //      warp (ties: least total so far, which rotates single columns)
    seq.assign(W, {});
    seqpos.assign(C.size(), 0);
    std::vector<double> tot(W, 0.0);
    for (int L = 0; L < NL; L++) {
      std::vector<int> cols = level_tasks(L);
      std::stable_sort(cols.begin(), cols.end(), [&](int a, int b) { return C[a].cost > C[b].cost; });
      std::vector<double> load(W, 0.0);
      std::vector<std::vector<int>> mine(W);
      for (int k : cols) {
        int best = 0;
        // a column whose block leaves less than two update pieces of room in
        // a regular ring runs on warp 0 (whose ring is larger when the plan
        // has such columns)
        if (P.big_rows <= R || C[k].brows <= R - 2 * kPieceRows)
          for (int w = 1; w < W; w++)
            if (load[w] < load[best] || (load[w] == load[best] && tot[w] < tot[best])) best = w;
        load[best] += C[k].cost;
        tot[best] += C[k].cost;
        C[k].warp = best;
        mine[best].push_back(k);
      }
      for (int w = 0; w < W; w++)
        for (int k : mine[w]) {
          seqpos[k] = (int)seq[w].size();
          seq[w].push_back(k);
        }
    }
    // ---- columns of narrow levels run in slices at earlier levels
    for (int L = 2; L < NR; L++) {
      const int width = sc.lev_ptr[L + S0 + 1] - sc.lev_ptr[L + S0];
      if (width > std::max(1, W / 4)) continue;
      for (int q = sc.lev_ptr[L + S0]; q < sc.lev_ptr[L + S0 + 1]; q++) {
        ColInfo& c = C[sc.lev_cols[q]];
        c.run_early.assign(c.nlr, 0);
        int e = 0;
        for (int r = 0; r < c.nlr; r++) {
          e = std::max(e, C[c.items[r].j].level + 1);
          c.run_early[r] = e;
        }
        const int nfw = ((int)c.items.size() - c.nlr) / 2;
        c.fw_early.assign(nfw, 0);
        e = 0;
        for (int f = 0; f < nfw; f++) {
          e = std::max(e, std::max(C[c.items[c.nlr + 2 * f].j].level,
                                   C[c.items[c.nlr + 2 * f + 1].j].level) + 1);
          c.fw_early[f] = e;
        }
        c.split = with_pre && ((c.nlr > 0 && c.run_early[0] < L) || (nfw > 0 && c.fw_early[0] < L));
      }
    }
    // ---- simulate the warps level by level and emit
    busy.assign((size_t)T, -1);
    tag.assign((size_t)T, -1);
    cursor.assign(W, 0);
    ngroups.assign(W, 0);
    waited.assign(W, -1);
    pos.assign(W, 0);
    em.assign(W, Emit(P.chunk_words));
    uncommitted.assign(W, {});
    uncommitted_cols.assign(W, {});
    pend_rows.assign(W, {});
    last_colhdr.assign(W, -1);
    last_colend.assign(W, -1);
    wcost.assign(W, 0.0);
    pinned.assign(W, 0);
    hpend.assign(W, {});
    last_pub.assign(W, -1);
    if (P.sync && (!reqs || (int)reqs->size() != W)) {
      err = "progress flags without their analysis";
      return false;
    }
    std::vector<int> wnext(W, 0);
    for (int L = 0; L < NL; L++) {
      for (int w = 0; w < W; w++) { pos[w] = 0; pinned[w] = 0; }
      // stage blocks the warps' previous columns could not issue ahead are
      // placed first, before any value is pinned for reading in place
      for (int w = 0; w < W; w++) {
        const int q = wnext[w];
        if (q < (int)seq[w].size() && C[seq[w][q]].level == L && !C[seq[w][q]].staged)
          stage_col(w, seq[w][q], now(w, L));
      }
      // values finished at earlier levels that are still in some ring
      for (int id : level_tasks(L)) {
        ColInfo& c = C[id];
        for (Item& it : c.items)
          if (it.state == ST_NONE) try_resident(it, L);
      }
      // ... and of the slices the idle warps will run for their next columns
      for (int w = 0; w < W; w++) {
        if (wnext[w] < (int)seq[w].size() && C[seq[w][wnext[w]]].level == L) continue;  // busy
        const int nq = next_own(w, wnext[w], L);
        if (nq < 0) continue;
        ColInfo& c = C[seq[w][nq]];
        const Part pt = slice_part(c, L);
        for (size_t r = pt.r0; r < pt.r1; r++)
          if (c.items[r].state == ST_NONE) try_resident(c.items[r], L);
        for (size_t f = pt.f0; f < pt.f1; f++)
          if (c.items[f].state == ST_NONE) try_resident(c.items[f], L);
      }
      std::fill(wcost.begin(), wcost.end(), 0.0);
      std::vector<char> idle(W, 0);
      idle_warps.clear();
      bundles.clear();
      for (int w = 0; w < W; w++) {
        idle[w] = !(wnext[w] < (int)seq[w].size() && C[seq[w][wnext[w]]].level == L);
        if (idle[w] && with_helpers) idle_warps.push_back(w);
      }
      auto bar = [&](int w) {
        helper_wait(w, L);
        Emit& e = em[w];
        const bool rides = last_colhdr[w] >= 0 && last_colend[w] == (int64_t)e.w.size();
        const int64_t rides_at = last_colhdr[w];
        last_colhdr[w] = -1;
        if (P.sync == 0) {
          if (rides) {
            e.w[rides_at] |= (1 << 8);  // the level's barrier rides on the last column
          } else {
            e.need(1);
            e.w.push_back(CMD_BAR);
          }
          return;
        }
        // progress flags: L + 1 levels done, published by the last column or
        // by PUB (an idle stretch of levels takes one PUB, raised in place);
        // then the waits that open the warp's next level
        if (rides) {
          e.w[rides_at] |= (1 << 8);
          last_pub[w] = -1;
        } else if (last_pub[w] >= 0 && last_pub[w] + 1 == (int64_t)e.w.size()) {
          e.w[last_pub[w]] = CMD_PUB | ((L + 1) << 4);
        } else {
          e.need(1);
          last_pub[w] = (int64_t)e.w.size();
          e.w.push_back(CMD_PUB | ((L + 1) << 4));
        }
        if (L + 1 < NL) {
          const std::vector<int32_t>& rq = (*reqs)[w][L + 1];
          if (!rq.empty()) {
            e.need(1 + rq.size());
            e.w.push_back(CMD_WAITP | ((int32_t)rq.size() << 4));
            for (int32_t x : rq) e.w.push_back(x);
            out->n_waitp++;
            out->n_wait_reqs += (int64_t)rq.size();
          }
        }
      };
      for (int w = 0; w < W; w++) {
        if (idle[w]) continue;
        while (wnext[w] < (int)seq[w].size() && C[seq[w][wnext[w]]].level == L) {
          if (!run_col(w, seq[w][wnext[w]], L)) return false;
          wnext[w]++;
        }
        bar(w);
      }
      // the idle warps: shares of the helper copies (pairs of copies to the
      // warp with the least estimated work: its slice and its shares so
      // far), then a slice of their next column, then the waits due
      std::vector<double> load(W, 0.0);
      std::vector<int> slice_q(W, -1);
      for (int w : idle_warps) {
        const int nq = next_own(w, wnext[w], L);
        slice_q[w] = nq;
        if (nq < 0) continue;
        const ColInfo& c = C[seq[w][nq]];
        const Part pt = slice_part(c, L);
        size_t st = 0;
        for (size_t r = pt.r0; r < pt.r1; r++) st += (c.items[r].nrows + kStepOps - 1) / kStepOps;
        load[w] = part_empty(pt) ? 0.0 : 80 + step_cost() * st + fma_cost() * ((pt.f1 - pt.f0) / 2);
      }
      // shares[w]: per deadline, the rows warp w copies
      std::vector<std::vector<Bundle>> shares(W);
      const size_t q2 = 2 * (size_t)rpi();
      std::stable_sort(bundles.begin(), bundles.end(),
                       [](const Bundle& a, const Bundle& b) { return a.deadline < b.deadline; });
      for (Bundle& b : bundles) {
        for (size_t i = 0; i < b.rows.size(); i += q2) {
          int h = idle_warps[0];
          for (int x : idle_warps)
            if (load[x] < load[h]) h = x;
          load[h] += 140;
          std::vector<Bundle>& sh = shares[h];
          if (sh.empty() || sh.back().deadline != b.deadline) sh.push_back({{}, b.deadline});
          sh.back().rows.insert(sh.back().rows.end(), b.rows.begin() + i,
                                b.rows.begin() + std::min(b.rows.size(), i + q2));
        }
      }
      for (int w = 0; w < W; w++) {
        if (!idle[w]) continue;
        for (Bundle& sh : shares[w]) helper_gather(w, sh.rows, sh.deadline);
        const int nq = with_helpers ? slice_q[w] : next_own(w, wnext[w], L);
        if (nq >= 0) run_slice(w, seq[w][nq], L);
        bar(w);
      }
      st.est_cycles += *std::max_element(wcost.begin(), wcost.end()) + 120;
    }
    st.n_levels = NL;
    st.n_bars = P.sync ? 0 : NL;
    st.has_bwd = with_bwd;
    // ---- assemble
    st.chunk0.assign(W, 0);
    st.nchunks.assign(W, 0);
    for (int w = 0; w < W; w++) {
      Emit& e = em[w];
      e.w.push_back(CMD_END);
      while (e.w.size() < e.cstart + e.cw) e.w.push_back(CMD_NOP);
      st.chunk0[w] = (int32_t)(st.words.size() / P.chunk_words);
      st.nchunks[w] = (int32_t)(e.w.size() / P.chunk_words);
      st.words.insert(st.words.end(), e.w.begin(), e.w.end());
    }
    return true;
  }
};

}  // namespace

static bool choose_stream_1(const Schedule& sc, int elem, size_t smem_budget, Stream& out,
                            std::string& why, bool with_bwd, int sync, int wl, int wp, int wr,
                            int wmin);

using WaitLists = std::vector<std::vector<std::vector<int32_t>>>;
static std::string interpret(const Schedule& sc, const Stream& st, std::vector<double>& lu,
                             const std::vector<double>& rhs, std::vector<double>& X,
                             bool& singular, WaitLists* reqs);

bool build_stream(const Schedule& sc, const StreamPlan& plan, Stream& out, std::string& why,
                  bool with_bwd) {
  WaitLists reqs;
  if (plan.sync) {
    // the barrier form of the same schedule, run through the interpreter to
    // find each level's waits; the flag form is then emitted with them (the
    // builder makes the same decisions for both: no placement depends on
    // where commands fall in the stream chunks)
    StreamPlan pb = plan;
    pb.sync = 0;
    Stream sb;
    if (!build_stream(sc, pb, sb, why, with_bwd)) return false;
    std::vector<double> lu(sc.n_slots, 1.0), rhs(sc.n_u, 0.0), X;
    bool sing = false;
    const std::string e = interpret(sc, sb, lu, rhs, X, sing, &reqs);
    if (!e.empty()) {
      why = "progress-flag analysis: " + e;
      return false;
    }
  }
  Builder b(sc, plan);
  b.with_bwd = with_bwd;
  if (plan.sync) b.reqs = &reqs;
  bool ok = false;
  try {
    ok = b.build(out);
  } catch (const std::exception& e) {
    b.err = e.what();
    ok = false;
  }
  if (!ok) why = b.err;
  return ok;
}

bool choose_stream(const Schedule& sc, int elem, size_t smem_budget, Stream& out,
                   std::string& why, int sync, int wide_min) {
  // with the wide kernels' split when asked and the schedule has one, then
  // with the backward substitution in the stream when the schedule allows
  // it (no off-diagonal BTF entries), else (or when no plan holds it) without
  int wl = 0, wp = 0, wr = 0;
  wide_split(sc, wide_min, wl, wp, wr);
  if (wl + wp > 0 && choose_stream_1(sc, elem, smem_budget, out, why, true, sync, wl, wp, wr, wide_min))
    return true;
  for (bool bwd : {sc.fuse_fwd, false}) {
    if (choose_stream_1(sc, elem, smem_budget, out, why, bwd, sync, 0, 0, 0, 0)) return true;
    if (!bwd) break;
  }
  return false;
}

// The plan with nw warps and chunk_words-word stream chunks in the budget:
// the rest of the shared memory split into rings (one larger ring for warp 0
// when some column's block does not fit an even share).  False when none.
static bool plan_for(const Schedule& sc, int elem, size_t smem_budget, int nw, int chunk_words,
                     StreamPlan& p) {
  int max_brows = 1;
  for (int k = 0; k < sc.n_u; k++) max_brows = std::max(max_brows, sc.c_ulen[k] + 1 + sc.c_llen[k] + 3);
  p = StreamPlan{};
  p.elem = elem;
  p.nw = nw;
  p.chunk_words = chunk_words;
  const size_t fixed = (size_t)nw * 2 * p.chunk_words * 4 + (size_t)kSpareRows * 32 * elem;
  if (fixed >= smem_budget) return false;
  const int total = std::min((int)((smem_budget - fixed) / ((size_t)32 * elem)), kMaxRows - kSpareRows);
  int r = total / nw;
  int big = 0;
  if (max_brows > r && nw > 1) {
    // one large ring (warp 0) for the columns the even split cannot hold
    big = max_brows + max_brows / 8;
    r = (total - big) / (nw - 1);
    if (r < 32 || big <= r) return false;
  }
  if (r < 16) return false;
  p.ring_rows = r;
  p.big_rows = big;
  return true;
}

void wide_split(const Schedule& sc, int min_width, int& levels, int& phases, int& rows) {
  levels = phases = rows = 0;
  if (!sc.fuse_fwd || min_width <= 0) return;
  for (; levels < sc.n_levels - 1; levels++) {
    if (sc.lev_ptr[levels + 1] - sc.lev_ptr[levels] < min_width) break;
    int longest = 0;
    for (int q = sc.lev_ptr[levels]; q < sc.lev_ptr[levels + 1]; q++) {
      const int k = sc.lev_cols[q];
      longest = std::max(longest, sc.c_ulen[k] + 1 + sc.c_llen[k]);
    }
    if (longest > kWideCap) break;
    rows = std::max(rows, longest);
  }
  phases = levels;  // the rows of those columns, in reverse level order
}

std::vector<StreamPlan> candidate_plans(const Schedule& sc, int elem, size_t smem_budget) {
  std::vector<StreamPlan> out;
  int wl[2], wp[2], wr[2];
  wide_split(sc, kWideMinWidth, wl[0], wp[0], wr[0]);
  wide_split(sc, kWideMinWidthDeep, wl[1], wp[1], wr[1]);
  for (int nw : {12, 10, 8, 7, 6, 5}) {
    if (nw > (elem == 4 ? kMaxRefactorWarps : 8)) continue;
    for (int cw : {320, 512}) {
      StreamPlan p;
      if (!plan_for(sc, elem, smem_budget, nw, cw, p)) continue;
      for (int wide : {0, 1, 2}) {
        const int v = wide - 1;
        if (wide && wl[v] == 0) continue;
        if (wide == 2 && wl[1] == wl[0]) continue;  // the same split
        p.wide_levels = wide ? wl[v] : 0;
        p.wide_phases = wide ? wp[v] : 0;
        p.wide_rows = wide ? wr[v] : 0;
        p.wide_min = wide == 0 ? 0 : wide == 1 ? kWideMinWidth : kWideMinWidthDeep;
        for (int sync : {0, 1}) {
          if (wide == 2 && sync == 1) continue;  // the deep split with barriers only
          p.sync = sync;
          out.push_back(p);
        }
      }
    }
  }
  return out;
}

bool build_plan(const Schedule& sc, const StreamPlan& p, Stream& out, std::string& why) {
  if (p.wide_levels > 0 || p.wide_phases > 0) return build_stream(sc, p, out, why, true);
  for (bool bwd : {sc.fuse_fwd, false}) {
    if (build_stream(sc, p, out, why, bwd)) return true;
    if (!bwd) break;
  }
  return false;
}

static bool choose_stream_1(const Schedule& sc, int elem, size_t smem_budget, Stream& out,
                            std::string& why, bool with_bwd, int sync, int wl, int wp, int wr,
                            int wmin) {
  bool found = false;
  std::string last;
  for (int nw : {12, 10, 8, 6, 4, 3, 2, 1}) {
    if (nw > (elem == 4 ? kMaxRefactorWarps : 8)) continue;
    StreamPlan p;
    if (!plan_for(sc, elem, smem_budget, nw, nw >= 10 ? 320 : 512, p)) continue;
    p.sync = sync;
    p.wide_levels = wl;
    p.wide_phases = wp;
    p.wide_rows = wr;
    p.wide_min = wl > 0 ? wmin : 0;
    Stream s;
    std::string w;
    if (!build_stream(sc, p, s, w, with_bwd)) {
      last = w;
      continue;
    }
    out = std::move(s);
    found = true;
    break;  // the most warps that fit
  }
  if (!found) why = last.empty() ? "no plan fits the shared-memory budget" : last;
  return found;
}

// ---------------------------------------------------------------------------
// host interpreter

std::string run_stream_host(const Schedule& sc, const Stream& st, std::vector<double>& lu,
                            const std::vector<double>& rhs, std::vector<double>& X,
                            bool& singular) {
  return interpret(sc, st, lu, rhs, X, singular, nullptr);
}

// The interpreter proper.  With `reqs` it analyses a barrier-form stream:
// barriers order nothing, and every access that conflicts with an earlier
// one of another warp not yet ordered before it adds a wait to the warp's
// current level (reqs[w][L]: words v | n << 8), as the flag form will.
static std::string interpret(const Schedule& sc, const Stream& st, std::vector<double>& lu,
                             const std::vector<double>& rhs, std::vector<double>& X,
                             bool& singular, WaitLists* reqs) {
  const StreamPlan& P = st.plan;
  const int W = P.nw, CW = P.chunk_words, n = sc.n_u;
  const int T = ring_total(P);
  const int rows = T + kSpareRows;
  const int zero_row = T, trash_row = T + 1;
  const int rpi2 = 2 * (512 / (32 * P.elem));
  const int NLv = st.n_levels;
  std::vector<double> ring(rows, 0.0);
  std::vector<int> pend(rows, -1);  // commit group of a copy not yet waited for
  std::vector<int> col_of_slot(sc.n_slots, -1);
  for (int k = 0; k < n; k++)
    for (int p = 0; p < sc.c_ulen[k] + 1 + sc.c_llen[k]; p++) col_of_slot[sc.c_base[k] + p] = k;
  std::vector<int> colfin(n, -1), xfin(n, -1), bfin(n, -1);  // level of FINISH / BWD
  singular = false;
  if ((int)lu.size() != sc.n_slots || (int)rhs.size() != n) return "buffer sizes";
  if (NLv <= 0 || NLv >= 32000) return "level count out of range";
  X.assign(n, 0.0);
  // ---- the wide kernels' part before the stream: the columns of the first
  //      wide_levels levels, each as the wide kernel computes it (KLU's
  //      update order, the forward term, pivot and scaling), finished
  //      before level 0 of the stream (-2)
  const int S0 = P.wide_levels, PW = P.wide_phases;
  if (S0 < 0 || S0 >= sc.n_levels || PW != S0 || (S0 > 0 && !(sc.fuse_fwd && st.has_bwd)))
    return "bad wide split";
  for (int L = 0; L < S0; L++)
    for (int q = sc.lev_ptr[L]; q < sc.lev_ptr[L + 1]; q++) {
      const int k = sc.lev_cols[q], base = sc.c_base[k], ulen = sc.c_ulen[k];
      const int len = ulen + 1 + sc.c_llen[k];
      if (len > P.wide_rows || len > kWideCap) return "a wide-kernel column longer than its stage";
      std::vector<double> stg(lu.begin() + base, lu.begin() + base + len);
      for (int p = 0; p < ulen; p++) {
        const int e = sc.cu_ptr[k] + p, j = sc.cu_j[e];
        if (sc.col_level[j] >= L) return "a wide-kernel column reads one of its own level";
        const double x = stg[p];
        const int lb = sc.c_base[j] + sc.c_ulen[j] + 1;
        for (int i = 0; i < sc.c_llen[j]; i++) stg[sc.cu_dst[sc.cu_dptr[e] + i]] -= lu[lb + i] * x;
      }
      double y = rhs[k];
      for (int tt = sc.fw_ptr[k]; tt < sc.fw_ptr[k + 1]; tt++) y -= lu[sc.fw_slot[tt]] * X[sc.fw_col[tt]];
      if (stg[ulen] == 0.0) singular = true;
      const double inv = 1.0 / stg[ulen];
      for (int p = 0; p <= ulen; p++) lu[base + p] = stg[p];
      for (int p = ulen + 1; p < len; p++) lu[base + p] = stg[p] * inv;
      X[k] = y;
      colfin[k] = xfin[k] = -2;
    }
  // ---- happens-before between warps (progress-flag plans and the analysis)
  const bool flags = P.sync != 0, analyze = reqs != nullptr;
  const bool vcs = flags || analyze;
  if (flags && analyze) return "analysis of a stream that already has progress flags";
  // vc[w][v]: levels of warp v known to warp w to be done; pubvc[v][p]: v's
  // clock when it had published p levels; per access key (ring rows, then
  // factor slots and solution rows in global memory): the last writer and
  // its level, and per warp the last level it read the key since
  const int K = rows + sc.n_slots + n;
  std::vector<int> vc, pubvc, published(W, 0), lw_w, lw_l;
  std::vector<int16_t> rdl;
  if (vcs) {
    vc.assign((size_t)W * W, 0);
    pubvc.assign((size_t)W * (NLv + 1) * W, 0);
    lw_w.assign(K, -1);
    lw_l.assign(K, -1);
    rdl.assign((size_t)K * W, -1);
  }
  if (analyze) reqs->assign(W, std::vector<std::vector<int32_t>>(NLv));
  auto join = [&](int w, int v, int p) {
    const int* src = &pubvc[((size_t)v * (NLv + 1) + p) * W];
    for (int u = 0; u < W; u++) vc[(size_t)w * W + u] = std::max(vc[(size_t)w * W + u], src[u]);
  };
  auto publish = [&](int w, int p) {
    if (!vcs) return;
    vc[(size_t)w * W + w] = p;
    for (int q = published[w] + 1; q <= p; q++)
      std::copy(&vc[(size_t)w * W], &vc[(size_t)w * W] + W, &pubvc[((size_t)w * (NLv + 1) + q) * W]);
    published[w] = std::max(published[w], p);
  };
  // warp w, in level L, needs warp v's first p levels done
  std::string vce;
  auto need = [&](int w, int L, int v, int p) -> bool {
    if (v == w || p <= 0 || vc[(size_t)w * W + v] >= p) return true;
    if (p > L) {
      vce = "conflicts with warp " + std::to_string(v) + " within level " + std::to_string(L);
      return false;
    }
    if (!analyze) {
      vce = "conflicts with warp " + std::to_string(v) + "'s level " + std::to_string(p - 1) +
            " without a wait for it";
      return false;
    }
    if (published[v] < p) {
      vce = "depends on a level of warp " + std::to_string(v) + " not yet published";
      return false;
    }
    std::vector<int32_t>& rq = (*reqs)[w][L];
    bool found = false;
    for (int32_t& x : rq)
      if ((x & 0xff) == v) {
        x = v | (std::max(x >> 8, p) << 8);
        found = true;
      }
    if (!found) rq.push_back(v | (p << 8));
    join(w, v, p);
    return true;
  };
  auto acc_r = [&](int key, int w, int L) -> bool {
    if (!vcs) return true;
    if (lw_w[key] >= 0 && !need(w, L, lw_w[key], lw_l[key] + 1)) return false;
    int16_t& r = rdl[(size_t)key * W + w];
    if (r < L) r = (int16_t)L;
    return true;
  };
  auto acc_w = [&](int key, int w, int L) -> bool {
    if (!vcs) return true;
    if (lw_w[key] >= 0 && !need(w, L, lw_w[key], lw_l[key] + 1)) return false;
    for (int v = 0; v < W; v++) {
      int16_t& r = rdl[(size_t)key * W + v];
      if (r >= 0 && !need(w, L, v, r + 1)) return false;
    }
    for (int v = 0; v < W; v++) rdl[(size_t)key * W + v] = -1;
    lw_w[key] = w;
    lw_l[key] = L;
    return true;
  };
  const int gkey = rows;               // factor slot s: gkey + s
  const int xkey = rows + sc.n_slots;  // solution row k: xkey + k
  struct WS {
    int chunk = 0, pc = 0, ng = 0, bars = 0;
    bool done = false;
    std::vector<int> pend_rows;
  };
  std::vector<WS> ws(W);
  for (int w = 0; w < W; w++) ws[w].pc = st.chunk0[w] * CW;
  // per level: who touched which row
  std::vector<int> wr_by(rows, -1), rd_by(rows, -1), stamp_w(rows, -1), stamp_r(rows, -1);
  for (int L = 0; L <= NLv; L++) {
    for (int w = 0; w < W; w++) {
      WS& s = ws[w];
      if (s.done || s.bars > L) continue;  // finished, or already past this level's barrier
      std::string e;
      auto fail = [&](const std::string& m) {
        return "warp " + std::to_string(w) + " word " + std::to_string(s.pc) + " (op " +
               std::to_string(st.words[s.pc] & 15) + "): " + m;
      };
      auto in_ring = [&](int r) { return r >= 0 && r < T; };
      auto note_w = [&](int r) -> bool {
        if (r == zero_row) { e = "writes the zero row"; return false; }
        if (pend[r] >= 0) { e = "row " + std::to_string(r) + " written while a copy into it is in flight"; return false; }
        if (!acc_w(r, w, L)) { e = vce + " (row " + std::to_string(r) + ")"; return false; }
        if (stamp_w[r] == L && wr_by[r] != w) { e = "two warps write row " + std::to_string(r); return false; }
        if (stamp_r[r] == L && rd_by[r] != w) {
          e = "row " + std::to_string(r) + " written while warp " + std::to_string(rd_by[r]) +
              " reads it (level " + std::to_string(L) + ")";
          return false;
        }
        stamp_w[r] = L;
        wr_by[r] = w;
        return true;
      };
      auto note_r = [&](int r) -> bool {
        if (pend[r] >= 0) { e = "row " + std::to_string(r) + " read before its copy is waited for"; return false; }
        if (!acc_r(r, w, L)) { e = vce + " (row " + std::to_string(r) + ")"; return false; }
        if (stamp_w[r] == L && wr_by[r] != w) {
          e = "row " + std::to_string(r) + " read while warp " + std::to_string(wr_by[r]) +
              " writes it (level " + std::to_string(L) + ")";
          return false;
        }
        if (stamp_r[r] == L && rd_by[r] != w) rd_by[r] = -2;
        else if (stamp_r[r] != L) { stamp_r[r] = L; rd_by[r] = w; }
        return true;
      };
      const int cbeg = (st.chunk0[w] + s.chunk) * CW;
      auto gather = [&](int at, int m, bool commit) -> bool {
        if (m % rpi2) { e = "gather list not padded"; return false; }
        for (int q = 0; q < m; q++) {
          const uint32_t rw = (uint32_t)st.words[at + q];
          const int src = (int)(rw & 0x1fffff), dst = (int)(rw >> 21);
          if (dst == trash_row && src == 0) continue;  // padding copy
          // (into any warp's ring: an idle warp copies for another warp's
          // next task, and the race checks below cover the sharing)
          if (dst < 0 || dst >= T) { e = "gather outside the rings"; return false; }
          if (pend[dst] >= 0) { e = "gather onto a row with a copy in flight"; return false; }
          double v;
          if (src < sc.n_slots) {
            const int col = col_of_slot[src];
            if (colfin[col] >= L) { e = "copies a value finished in the same level"; return false; }
            v = lu[src];
          } else if (src < sc.n_slots + n) {
            const int r = src - sc.n_slots;
            if (bfin[r] >= 0 ? bfin[r] >= L : (xfin[r] == -1 || xfin[r] >= L)) {
              e = "copies X before its value is final";
              return false;
            }
            v = X[r];
          } else if (src < sc.n_slots + 2 * n) {
            v = rhs[src - sc.n_slots - n];
          } else {
            e = "source row out of range";
            return false;
          }
          if (src < sc.n_slots + n && !acc_r(gkey + src, w, L)) {
            e = vce + " (global row " + std::to_string(src) + ")";
            return false;
          }
          if (!note_w(dst)) return false;
          ring[dst] = v;
          pend[dst] = s.ng;
          s.pend_rows.push_back(dst);
        }
        if (commit) s.ng++;
        return true;
      };
      auto wait = [&](int m) {
        const int upto = s.ng - 1 - m;
        std::vector<int> keep;
        for (int r : s.pend_rows) {
          if (pend[r] >= 0 && pend[r] <= upto) {
            pend[r] = -1;
            if (vcs) lw_l[r] = L;  // the copy's write is complete from here on
          }
          if (pend[r] >= 0) keep.push_back(r);
        }
        s.pend_rows.swap(keep);
      };
      auto steps = [&](int first, int m, int S0) -> bool {
        if (m % 2) { e = "odd step count"; return false; }
        if (first + 4 * m + 8 > cbeg + CW) { e = "steps past the chunk"; return false; }
        for (int q = 0; q < m; q++) {
          const uint32_t* d = reinterpret_cast<const uint32_t*>(&st.words[first + 4 * q]);
          const int lrow = (int)(d[0] & 0xffff), jp = (int)((d[0] >> 16) & 0x3ff), cnt = (int)(d[0] >> 26);
          if (cnt > kStepOps) { e = "bad step count"; return false; }
          if (lrow + kStepOps > rows) { e = "step L rows out of range"; return false; }
          if (!in_ring(S0 + jp)) { e = "step pivot row out of range"; return false; }
          const uint32_t dw[3] = {d[1], d[2], d[3]};
          for (int tt = cnt; tt < kStepOps; tt++) {
            const int ur = S0 + (int)((dw[tt / 3] >> (10 * (tt % 3))) & 0x3ff);
            if (!in_ring(ur)) {
              e = "unused step slot outside the ring";
              return false;
            }
            // FP32 steps run all nine updates: the unused ones write their
            // (dummy) row, which another warp may copy into later
            if (P.elem == 4 && !note_w(ur)) return false;
          }
          if (cnt == 0) continue;  // padding step
          if (!note_r(S0 + jp)) return false;
          const double xj = ring[S0 + jp];
          for (int tt = 0; tt < cnt; tt++) {
            const int dr = S0 + (int)((dw[tt / 3] >> (10 * (tt % 3))) & 0x3ff);
            if (!in_ring(dr) || !in_ring(lrow + tt)) { e = "step row out of range"; return false; }
            if (dr == S0 + jp) { e = "step writes its pivot row"; return false; }
            if (!note_r(lrow + tt) || !note_r(dr) || !note_w(dr)) return false;
            ring[dr] = ring[dr] - ring[lrow + tt] * xj;
          }
        }
        return true;
      };
      auto fwd = [&](int at, int m, bool first, int S0, int len) -> bool {
        if (!sc.fuse_fwd) { e = "forward terms without fusion"; return false; }
        if (m % 8) { e = "forward terms not padded"; return false; }
        if (!in_ring(S0 + len + 1)) { e = "forward rows out of range"; return false; }
        const int yr0 = S0 + len;
        if (!note_r(first ? yr0 + 1 : yr0)) return false;
        double y = ring[first ? yr0 + 1 : yr0];
        for (int f = 0; f < m; f++) {
          const uint32_t fw = (uint32_t)st.words[at + f];
          const int lr = (int)(fw & 0xffff), yr = (int)(fw >> 16);
          if (lr == zero_row && yr == zero_row) continue;  // padding term
          if (!in_ring(lr) || !in_ring(yr)) { e = "forward term row out of range"; return false; }
          if (!note_r(lr) || !note_r(yr)) return false;
          y -= ring[lr] * ring[yr];
        }
        if (!note_w(yr0)) return false;
        ring[yr0] = y;
        return true;
      };
      auto finish = [&](int k, int base, int ulen, int llen, int S0) -> bool {
        const int len = ulen + 1 + llen;
        if (k < 0 || k >= n || base != sc.c_base[k] || ulen != sc.c_ulen[k] || llen != sc.c_llen[k]) {
          e = "FINISH header does not match the column";
          return false;
        }
        if (!in_ring(S0) || !in_ring(S0 + len + 2) || ring_warp(P, S0) != w ||
            ring_warp(P, S0 + len + 2) != w) {
          e = "stage block out of range";
          return false;
        }
        for (int p = 0; p < len; p++)
          if (!note_r(S0 + p)) return false;
        const double piv = ring[S0 + ulen];
        if (piv == 0.0) singular = true;
        const double inv = 1.0 / piv;
        for (int p = 0; p < len; p++)
          if (!acc_w(gkey + base + p, w, L)) {
            e = vce + " (factor slot " + std::to_string(base + p) + ")";
            return false;
          }
        for (int p = 0; p <= ulen; p++) lu[base + p] = ring[S0 + p];
        for (int p = ulen + 1; p < len; p++) {
          if (!note_w(S0 + p)) return false;
          ring[S0 + p] = ring[S0 + p] * inv;
          lu[base + p] = ring[S0 + p];
        }
        colfin[k] = L;
        if (sc.fuse_fwd) {
          if (!note_r(S0 + len)) return false;
          if (!acc_w(xkey + k, w, L)) {
            e = vce + " (solution row " + std::to_string(k) + ")";
            return false;
          }
          X[k] = ring[S0 + len];
          xfin[k] = L;
        }
        return true;
      };
      // the end of this warp's work of level L (a barrier, or its progress
      // flag), and the level count it has then done
      auto level_end = [&](int p) -> bool {
        if (p <= s.bars || p > NLv) { e = "level count " + std::to_string(p) + " out of order"; return false; }
        s.bars = p;
        publish(w, p);
        return true;
      };
      for (;;) {
        const int cend = (st.chunk0[w] + s.chunk + 1) * CW - 1;  // NEXT / END word
        if (s.pc < cbeg || s.pc > cend) return fail("ran past its chunk");
        const int32_t w0 = st.words[s.pc];
        const int op = w0 & 15;
        if (op == CMD_NOP) { s.pc++; continue; }
        if (op == CMD_NEXT) {
          if (++s.chunk >= st.nchunks[w]) return fail("NEXT past the last chunk");
          s.pc = (st.chunk0[w] + s.chunk) * CW;
          break;  // re-enter with the new chunk bounds
        }
        if (op == CMD_END) {
          if (s.bars != NLv) return fail("END after a wrong number of levels");
          s.done = true;
          break;
        }
        if (op == CMD_BAR) {
          if (flags) return fail("a barrier in a plan with progress flags");
          if (!level_end(s.bars + 1)) return fail(e);
          s.pc++;
          break;
        }
        if (op == CMD_PUB) {
          if (!flags) return fail("a progress flag in a plan with barriers");
          if (!level_end((int)(((uint32_t)w0) >> 4))) return fail(e);
          s.pc++;
          break;
        }
        if (op == CMD_WAITP) {
          if (!flags) return fail("a progress-flag wait in a plan with barriers");
          const int m = (w0 >> 4) & 0xff;
          if (m < 1 || m >= W || s.pc + 1 + m > cend) return fail("bad WAITP command");
          for (int q = 0; q < m; q++) {
            const int32_t x = st.words[s.pc + 1 + q];
            const int v = x & 0xff, p = (int)(((uint32_t)x) >> 8);
            if (v >= W || v == w || p < 1 || p > s.bars) return fail("bad WAITP entry");
            // in level order every level waited for is published first, so
            // no warp waits for one that can only come after its own wait
            if (published[v] < p) return fail("waits for a level not yet published");
            join(w, v, p);
          }
          s.pc += 1 + m;
          continue;
        }
        if (op == CMD_GATHER) {
          const int m = (w0 >> 4) & 0xffff;
          if (s.pc + 1 + m > cend) return fail("GATHER past its chunk");
          if (!gather(s.pc + 1, m, (w0 >> 23) & 1)) return fail(e);
          s.pc += 1 + m;
          continue;
        }
        if (op == CMD_WAIT) { wait((w0 >> 4) & 7); s.pc++; continue; }
        if (op == CMD_STEPS) {
          const int m = (w0 >> 4) & 0xfff, S0 = (int)(((uint32_t)w0) >> 16);
          const int first = (s.pc + 1 + 3) & ~3;
          if (!steps(first, m, S0)) return fail(e);
          s.pc = first + 4 * m;
          continue;
        }
        if (op == CMD_FWD) {
          const int m = (w0 >> 4) & 0xffff;
          const int S0 = st.words[s.pc + 1] & 0xffff, len = (st.words[s.pc + 1] >> 16) & 0xffff;
          if (s.pc + 2 + m > cend) return fail("FWD past its chunk");
          if (!fwd(s.pc + 2, m, (w0 >> 20) & 1, S0, len)) return fail(e);
          s.pc += 2 + m;
          continue;
        }
        if (op == CMD_FINISH) {
          if (s.pc + 5 > cend) return fail("FINISH past its chunk");
          const int ul = st.words[s.pc + 3];
          if (!finish(st.words[s.pc + 1], st.words[s.pc + 2], ul & 0xffff, (ul >> 16) & 0xffff,
                      st.words[s.pc + 4]))
            return fail(e);
          s.pc += 5;
          continue;
        }
        if (op == CMD_BWD) {
          if (s.pc + 5 > cend) return fail("BWD header past its chunk");
          const int k = st.words[s.pc + 1];
          const uint32_t w2 = (uint32_t)st.words[s.pc + 2], w3 = (uint32_t)st.words[s.pc + 3];
          const uint32_t w4 = (uint32_t)st.words[s.pc + 4];
          const int xr = (int)(w2 & 0xffff), yr = (int)(w2 >> 16), dr = (int)(w3 & 0xffff);
          const int m = (int)(w3 >> 16), nl = (int)(w4 & 0xffff), np = (int)(w4 >> 16);
          const int mr = (int)(((uint32_t)w0) >> 20);
          if (!st.has_bwd || k < 0 || k >= n) return fail("bad BWD command");
          if (s.pc + 5 + nl + np + m > cend) return fail("BWD past its chunk");
          if (m % 8 || mr > m) return fail("BWD terms not padded");
          if (nl && !gather(s.pc + 5, nl, true)) return fail(e);
          if (np && !gather(s.pc + 5 + nl, np, true)) return fail(e);
          if ((w0 >> 7) & 1) wait((w0 >> 4) & 7);
          if (!in_ring(xr) || ring_warp(P, xr) != w || !in_ring(yr) || !in_ring(dr))
            return fail("BWD rows out of range");
          if (!note_r(yr) || !note_r(dr)) return fail(e);
          double v = ring[yr];
          const int tb = s.pc + 5 + nl + np;
          for (int f = 0; f < m; f++) {
            const uint32_t fw = (uint32_t)st.words[tb + f];
            const int ur = (int)(fw & 0xffff), xj = (int)(fw >> 16);
            if (ur == zero_row && xj == zero_row) {
              if (f < mr) return fail("padding inside the real BWD terms");
              continue;
            }
            if (f >= mr) return fail("BWD term after the real count");
            if (!in_ring(ur) || !in_ring(xj)) return fail("BWD term row out of range");
            if (!note_r(ur) || !note_r(xj)) return fail(e);
            v -= ring[ur] * ring[xj];
          }
          const double x = v / ring[dr];
          if (!std::isfinite(x)) singular = true;
          if (!note_w(xr)) return fail(e);
          if (!acc_w(xkey + k, w, L)) return fail(vce + " (solution row " + std::to_string(k) + ")");
          ring[xr] = x;
          X[k] = x;
          bfin[k] = L;
          s.pc = tb + m;
          if ((w0 >> 8) & 1) {
            if (!level_end(s.bars + 1)) return fail(e);
            break;
          }
          continue;
        }
        if (op == CMD_COLUMN) {
          if (s.pc + 8 > cend) return fail("COLUMN header past its chunk");
          const int k = st.words[s.pc + 1], base = st.words[s.pc + 2], ul = st.words[s.pc + 3];
          const uint32_t h4 = (uint32_t)st.words[s.pc + 4], h5 = (uint32_t)st.words[s.pc + 5];
          const int nf = st.words[s.pc + 6];
          const int S0 = (int)(h4 & 0xffff), nl = (int)(h4 >> 16), np = (int)(h5 & 0xffff), ns = (int)(h5 >> 16);
          const int ulen = ul & 0xffff, llen = (ul >> 16) & 0xffff;
          const int sw = (s.pc + 8 + nl + np + 3) & ~3;
          if (sw + 4 * ns + nf > cend) return fail("COLUMN past its chunk");
          if (nl && !gather(s.pc + 8, nl, true)) return fail(e);
          if (np && !gather(s.pc + 8 + nl, np, true)) return fail(e);
          if ((w0 >> 7) & 1) wait((w0 >> 4) & 7);
          if (!steps(sw, ns, S0)) return fail(e);
          if (sc.fuse_fwd && !fwd(sw + 4 * ns, nf, !((w0 >> 9) & 1), S0, ulen + 1 + llen)) return fail(e);
          if (!sc.fuse_fwd && nf) return fail("forward terms without fusion");
          if (!((w0 >> 10) & 1) && !finish(k, base, ulen, llen, S0)) return fail(e);
          s.pc = sw + 4 * ns + nf;
          if ((w0 >> 8) & 1) {
            if (!level_end(s.bars + 1)) return fail(e);
            break;
          }
          continue;
        }
        return fail("bad opcode " + std::to_string(op));
      }
    }
    // warps that stopped at a chunk switch (NEXT) continue in this level
    bool again = false;
    for (int w = 0; w < W; w++)
      if (!ws[w].done && ws[w].bars <= L) again = true;
    if (again) L--;
  }
  for (int w = 0; w < W; w++)
    if (!ws[w].done) return "warp " + std::to_string(w) + " did not reach END";
  // ---- the wide kernels' part after the stream: the backward substitution
  //      of the wide columns' rows, one refactor level at a time from the
  //      last wide level down
  for (int L = PW - 1; L >= 0; L--)
    for (int q = sc.lev_ptr[L]; q < sc.lev_ptr[L + 1]; q++) {
      const int k = sc.lev_cols[q];
      double v = X[k];
      for (int tt = sc.bw_ptr[k]; tt < sc.bw_ptr[k + 1]; tt++) {
        const int j = sc.bw_col[tt];
        if (bfin[j] < 0) return "a wide-kernel row reads x of a row not yet solved";
        v -= lu[sc.bw_slot[tt]] * X[j];
      }
      const double x = v / lu[sc.diag_slot[k]];
      if (!std::isfinite(x)) singular = true;
      X[k] = x;
      bfin[k] = NLv;
    }
  for (int k = 0; k < n; k++)
    if (colfin[k] == -1) return "column " + std::to_string(k) + " never finished";
  if (st.has_bwd)
    for (int k = 0; k < n; k++)
      if (bfin[k] < 0) return "row " + std::to_string(k) + " of the backward substitution never solved";
  return "";
}

}  // namespace gox
