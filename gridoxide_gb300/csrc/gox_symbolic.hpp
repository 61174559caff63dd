// Host-side symbolic analysis for one topology: Jacobian pattern, CSC map,
// BTF + AMD ordering, and the first numeric factorization with partial
// pivoting that fixes the static pivot order the GPU refactors with.
//
// Everything here runs once per topology on the CPU.  Each piece reproduces
// the reference's (gridoxide's KluNative, and the SuiteSparse KLU C it was
// translated from) results exactly -- same permutations, same L/U patterns,
// same pivot rows -- because the batched GPU refactor reuses that static
// pivot order for every scenario.
#pragma once
#include <cstdint>
#include <vector>

namespace gox {

enum BusType : int32_t { BUS_PQ = 1, BUS_PV = 2, BUS_SLACK = 3 };

// The eight Jacobian entry kinds (gridoxide src/jacobian.rs:48-57).
enum JacKind : int32_t { K_HII = 0, K_NII = 1, K_HIK = 2, K_NIK = 3,
                         K_MII = 4, K_LII = 5, K_MIK = 6, K_LIK = 7 };

// JacobianPattern::analyze (src/jacobian.rs:96-171): entries in emission
// order -- H/N rows (non-slack buses, bus order, Y row ascending), then M/L
// rows (PQ buses).
struct JacPattern {
  int n_bus = 0, n_ang = 0, n_pq = 0, n_u = 0;
  std::vector<int32_t> rows, cols, kind, bi, bk, yslot;
  std::vector<int32_t> ns_idx, pq_idx;     // unknown -> bus
  std::vector<int32_t> ns_pos, pq_pos;     // bus -> unknown (or -1)
  int nnz() const { return (int)rows.size(); }
};
JacPattern jac_analyze(int n_bus, const int32_t* yp, const int32_t* yi, const int32_t* bus_type);

// build_csc_structure (src/klu_native/mod.rs:88-114): sort triplets by
// (col, row), merge duplicates.  slot_of[e] = CSC slot of triplet e.
struct Csc {
  int n = 0;
  std::vector<int32_t> p, i, slot_of;
  int nnz() const { return (int)i.size(); }
};
Csc build_csc(int n, int ntrip, const int32_t* rows, const int32_t* cols);

// BTF (btf_order: maxtrans + strongcomp).  Q may hold flipped columns when
// the matrix is structurally singular.
int btf_maxtrans(int n, const int32_t* Ap, const int32_t* Ai, int32_t* match);
int btf_strongcomp(int n, const int32_t* Ap, const int32_t* Ai, int32_t* Q, int32_t* P,
                   int32_t* R);
int btf_order(int n, const int32_t* Ap, const int32_t* Ai, int32_t* P, int32_t* Q, int32_t* R,
              int* nmatch);

// AMD ordering of the pattern of A + A' (dense 10, aggressive absorption).
// Returns 0 on success, <0 on invalid input.
int amd_order(int n, const int32_t* Ap, const int32_t* Ai, int32_t* perm);

// klu_analyze with BTF and AMD (src/klu_native/analyze.rs:67-150).
struct Symbolic {
  int n = 0, nblocks = 0, nmatch = 0;
  std::vector<int32_t> P, Q, R;
};
Symbolic klu_analyze(int n, const int32_t* Ap, const int32_t* Ai);

// First numeric factorization (KLU_kernel per block, tol 0.001, diagonal
// preference, Eisenstat-Liu pruning).  Patterns are stored per global
// column k in the KLU layout: U rows in the DFS (topological) order the
// refactor must follow, L rows in final pivot order; rows are global pivot
// positions.  Off holds the BTF off-diagonal entries, rows in pivot order.
struct Numeric {
  int n = 0;
  std::vector<int32_t> Pnum, Pinv;
  std::vector<int32_t> Lp, Li, Up, Ui;  // CSC, no diagonal; Lp/Up size n+1
  std::vector<double> Lx, Ux, Udiag;
  std::vector<int32_t> Offp, Offi;
  std::vector<double> Offx;
};
// Returns 0 ok, 1 singular.  vals: packed CSC values of A.
int klu_factor(const Csc& A, const double* vals, const Symbolic& S, double tol, Numeric& N);

}  // namespace gox
