"""ctypes front-end of the oracle -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module.  It wraps

* ``oracle/liboracle.so``: the plain-C restatement of the reference's
  batched Newton-Raphson path (see ``gox_oracle.h`` for the file:line map);
* ``oracle/_ref/libklu_ref.so`` (only where it was built): the reference's
  own vendored SuiteSparse KLU, driven through ``ref_shim.c``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libklu_ref.so")
# The reference checkout the recipe compiles from (its vendored SuiteSparse):
# $GRIDOXIDE_REFERENCE, else its default checkout location.
REF_ROOT = os.environ.get("GRIDOXIDE_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "vendor", "suitesparse")

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)


def build(ref: bool | None = None) -> None:
    """make -C oracle [ref]: the reference build only where its sources exist."""
    if ref is None:
        ref = os.path.isdir(REF_SRC)
    cmd = ["make", "-s", "-C", HERE]
    if ref:
        cmd += ["ref", f"REF={REF_SRC}"]
    subprocess.run(cmd, check=True)


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build(ref=False)
        L = C.CDLL(LIB)
        L.gxo_ybus_build.restype = C.c_int
        L.gxo_ybus_build.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p,
                                     _u8p, _i32p, _i32p, _f64p, _f64p]
        L.gxo_injections.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p, _f64p, _f64p]
        L.gxo_jac_analyze.restype = C.c_void_p
        L.gxo_jac_analyze.argtypes = [C.c_int, _i32p, _i32p, _i32p]
        L.gxo_jac_free.argtypes = [C.c_void_p]
        L.gxo_jac_nnz.restype = C.c_int
        L.gxo_jac_nnz.argtypes = [C.c_void_p]
        L.gxo_jac_nu.restype = C.c_int
        L.gxo_jac_nu.argtypes = [C.c_void_p]
        L.gxo_jac_pattern.argtypes = [C.c_void_p] + [_i32p] * 6
        L.gxo_jac_fill.argtypes = [C.c_void_p] + [_f64p] * 7
        L.gxo_lu_new.restype = C.c_void_p
        L.gxo_lu_new.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _i32p, _i32p, _i32p,
                                 C.c_int, C.POINTER(C.c_int)]
        L.gxo_lu_free.argtypes = [C.c_void_p]
        L.gxo_lu_factor_solve_values.restype = C.c_int
        L.gxo_lu_factor_solve_values.argtypes = [C.c_void_p, _f64p, _f64p, _f64p]
        L.gxo_lu_refactor.restype = C.c_int
        L.gxo_lu_refactor.argtypes = [C.c_void_p, _f64p]
        L.gxo_lu_solve.restype = C.c_int
        L.gxo_lu_solve.argtypes = [C.c_void_p, _f64p, _f64p]
        L.gxo_lu_sizes.argtypes = [C.c_void_p, _i32p]
        L.gxo_lu_extract.argtypes = [C.c_void_p, _i32p, _i32p, _f64p, _i32p, _i32p, _f64p,
                                     _i32p, _i32p, _f64p, _i32p, _i32p, _i32p]
        L.gxo_topo_new.restype = C.c_void_p
        L.gxo_topo_new.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _i32p, _i32p, _i32p,
                                   _i32p, C.c_int]
        L.gxo_topo_free.argtypes = [C.c_void_p]
        L.gxo_topo_set_zip.argtypes = [C.c_void_p, _f64p, _f64p, _f64p, _f64p]
        L.gxo_nr_solve.restype = C.c_int
        L.gxo_nr_solve.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), _f64p, _f64p, _f64p, _f64p,
                                   _f64p, _f64p, C.c_double, C.c_int, _f64p, C.POINTER(C.c_int)]
        L.gxo_batch_solve.restype = C.c_int
        L.gxo_batch_solve.argtypes = [C.c_void_p, C.c_int, _f64p, _f64p, _f64p, _f64p, C.c_int,
                                      _i32p, _f64p, _f64p, C.c_double, C.c_int, C.c_int,
                                      _f64p, _f64p, _i32p, _i32p, _f64p, _f64p]
        _lib = L
    return _lib


# ---------------------------------------------------------------------------
# building blocks

def ybus_build(g):
    """C restatement of the reference's Y-bus stamping for a grids.Grid."""
    L = lib()
    n, m = g.n_bus, g.n_branch
    cap = n + 4 * m + 1
    rp = np.zeros(n + 1, np.int32)
    ci = np.zeros(cap, np.int32)
    yr = np.zeros(cap)
    yi = np.zeros(cap)
    tr = np.ascontiguousarray(g.br_is_trafo, dtype=np.uint8)
    nnz = L.gxo_ybus_build(n, m, _p(_i32(g.br_from), _i32p), _p(_i32(g.br_to), _i32p),
                           _p(_f64(g.br_r), _f64p), _p(_f64(g.br_x), _f64p),
                           _p(_f64(g.br_b), _f64p), _p(_f64(g.br_tap), _f64p),
                           _p(tr, _u8p), _p(rp, _i32p), _p(ci, _i32p), _p(yr, _f64p),
                           _p(yi, _f64p))
    return rp, ci[:nnz].copy(), yr[:nnz].copy(), yi[:nnz].copy()


def injections(yb, vm, va):
    L = lib()
    n = yb.n
    p = np.zeros(n)
    q = np.zeros(n)
    L.gxo_injections(n, _p(_i32(yb.indptr), _i32p), _p(_i32(yb.indices), _i32p),
                     _p(_f64(yb.re), _f64p), _p(_f64(yb.im), _f64p), _p(_f64(vm), _f64p),
                     _p(_f64(va), _f64p), _p(p, _f64p), _p(q, _f64p))
    return p, q


class Jacobian:
    """JacobianPattern restatement (emission order, kinds, fill)."""

    def __init__(self, yb, bus_type):
        self.L = lib()
        self.yb = yb
        self._keep = (_i32(yb.indptr), _i32(yb.indices), _i32(bus_type))
        self.h = self.L.gxo_jac_analyze(yb.n, _p(self._keep[0], _i32p), _p(self._keep[1], _i32p),
                                        _p(self._keep[2], _i32p))
        self.nnz = self.L.gxo_jac_nnz(self.h)
        self.n_u = self.L.gxo_jac_nu(self.h)
        arrs = [np.zeros(self.nnz, np.int32) for _ in range(6)]
        self.L.gxo_jac_pattern(self.h, *[_p(a, _i32p) for a in arrs])
        self.rows, self.cols, self.kind, self.bi, self.bk, self.yslot = arrs

    def fill(self, vm, va, p, q, yre=None, yim=None):
        out = np.zeros(self.nnz)
        yre = self.yb.re if yre is None else yre
        yim = self.yb.im if yim is None else yim
        self.L.gxo_jac_fill(self.h, _p(_f64(yre), _f64p), _p(_f64(yim), _f64p),
                            _p(_f64(vm), _f64p), _p(_f64(va), _f64p), _p(_f64(p), _f64p),
                            _p(_f64(q), _f64p), _p(out, _f64p))
        return out

    def csc_pattern(self):
        """(Ap, Ai) of build_csc_structure."""
        n = self.n_u
        order = np.lexsort((self.rows, self.cols))
        ai = self.rows[order].astype(np.int32)
        ap = np.zeros(n + 1, np.int32)
        np.add.at(ap, self.cols[order] + 1, 1)
        return np.cumsum(ap).astype(np.int32), ai, order

    def __del__(self):
        try:
            self.L.gxo_jac_free(self.h)
        except Exception:
            pass


class LU:
    """KLU numeric restatement on a given ordering (P, Q, R)."""

    def __init__(self, n, rows, cols, vals, P, Q, R):
        self.L = lib()
        st = C.c_int(0)
        self.n = n
        self.h = self.L.gxo_lu_new(n, len(rows), _p(_i32(rows), _i32p), _p(_i32(cols), _i32p),
                                   _p(_f64(vals), _f64p), _p(_i32(P), _i32p), _p(_i32(Q), _i32p),
                                   _p(_i32(R), _i32p), len(R) - 1, C.byref(st))
        if not self.h:
            raise ZeroDivisionError("singular")

    def factor_solve(self, vals, rhs):
        x = np.zeros(self.n)
        bad = self.L.gxo_lu_factor_solve_values(self.h, _p(_f64(vals), _f64p),
                                                _p(_f64(rhs), _f64p), _p(x, _f64p))
        return None if bad else x

    def refactor(self, vals):
        return self.L.gxo_lu_refactor(self.h, _p(_f64(vals), _f64p))

    def extract(self):
        s = np.zeros(4, np.int32)
        self.L.gxo_lu_sizes(self.h, _p(s, _i32p))
        lnz, unz, nzoff, nb = [int(v) for v in s]
        n = self.n
        out = dict(Lp=np.zeros(n + 1, np.int32), Li=np.zeros(lnz, np.int32), Lx=np.zeros(lnz),
                   Up=np.zeros(n + 1, np.int32), Ui=np.zeros(unz, np.int32), Ux=np.zeros(unz),
                   Fp=np.zeros(n + 1, np.int32), Fi=np.zeros(max(nzoff, 1), np.int32),
                   Fx=np.zeros(max(nzoff, 1)), P=np.zeros(n, np.int32), Q=np.zeros(n, np.int32),
                   R=np.zeros(nb + 1, np.int32))
        self.L.gxo_lu_extract(self.h, *[_p(out[k], _i32p if out[k].dtype == np.int32 else _f64p)
                                        for k in ("Lp", "Li", "Lx", "Up", "Ui", "Ux", "Fp", "Fi",
                                                  "Fx", "P", "Q", "R")])
        out["Fi"] = out["Fi"][:nzoff]
        out["Fx"] = out["Fx"][:nzoff]
        return out

    def __del__(self):
        try:
            self.L.gxo_lu_free(self.h)
        except Exception:
            pass


class Topology:
    """Oracle topology: Y-bus + bus types + the Jacobian's symbolic ordering."""

    def __init__(self, yb, bus_type, P, Q, R):
        self.L = lib()
        self.n = yb.n
        self.yb = yb
        self.h = self.L.gxo_topo_new(yb.n, _p(_i32(yb.indptr), _i32p), _p(_i32(yb.indices), _i32p),
                                     _p(_f64(yb.re), _f64p), _p(_f64(yb.im), _f64p),
                                     _p(_i32(bus_type), _i32p), _p(_i32(P), _i32p),
                                     _p(_i32(Q), _i32p), _p(_i32(R), _i32p), len(R) - 1)

    def set_zip(self, imp=None, cur=None):
        """ZIP terms of effective_injection (src/network.rs:600-611): per bus
        a constant-impedance and a constant-current complex injection (per
        unit at |V| = 1); None clears both."""
        if imp is None and cur is None:
            self.L.gxo_topo_set_zip(self.h, None, None, None, None)
            return
        imp = np.zeros(self.n, np.complex128) if imp is None else np.asarray(imp, np.complex128)
        cur = np.zeros(self.n, np.complex128) if cur is None else np.asarray(cur, np.complex128)
        self._zip = [_f64(imp.real), _f64(imp.imag), _f64(cur.real), _f64(cur.imag)]
        self.L.gxo_topo_set_zip(self.h, *[_p(a, _f64p) for a in self._zip])

    def batch_solve(self, p_spec, q_spec, vm0, va0, tol=1e-8, max_iter=20, threads=1,
                    outage=None, history=False):
        """BatchSolver::solve restated.  p_spec/q_spec [B, N]; vm0/va0 [N] (shared)
        or [B, N]; outage = (slots [B,4], dre [B,4], dim [B,4]) or None."""
        p_spec = _f64(np.atleast_2d(p_spec))
        q_spec = _f64(np.atleast_2d(q_spec))
        B, n = p_spec.shape
        vm0 = _f64(vm0)
        va0 = _f64(va0)
        stride = n if vm0.ndim == 2 else 0
        vm = np.zeros((B, n))
        va = np.zeros((B, n))
        iters = np.zeros(B, np.int32)
        status = np.zeros(B, np.int32)
        mis = np.zeros(B)
        hist = np.zeros((B, max_iter)) if history else None
        if outage is not None:
            ds, dr, di = (_i32(outage[0]), _f64(outage[1]), _f64(outage[2]))
        else:
            ds = dr = di = None
        self.L.gxo_batch_solve(self.h, B, _p(p_spec, _f64p), _p(q_spec, _f64p), _p(vm0, _f64p),
                               _p(va0, _f64p), stride, _p(ds, _i32p), _p(dr, _f64p),
                               _p(di, _f64p), tol, max_iter, threads, _p(vm, _f64p),
                               _p(va, _f64p), _p(iters, _i32p), _p(status, _i32p),
                               _p(mis, _f64p), _p(hist, _f64p))
        res = dict(vm=vm, va=va, iters=iters, status=status, max_mis=mis)
        if history:
            res["hist"] = hist
        return res

    def __del__(self):
        try:
            self.L.gxo_topo_free(self.h)
        except Exception:
            pass


# ---------------------------------------------------------------------------
# the reference's orderings as committed fixtures (usable where the
# reference's KLU cannot be built)

GOLDEN = os.path.join(os.path.dirname(HERE), "tests", "golden")


def pattern_fingerprint(yb, bus_type) -> str:
    """sha256 of the Y-bus pattern and bus types: all the symbolic ordering
    of the Jacobian depends on."""
    import hashlib
    h = hashlib.sha256()
    for a in (yb.indptr, yb.indices, bus_type):
        h.update(np.ascontiguousarray(a, dtype="<i4").tobytes())
    return h.hexdigest()


def fixture_ordering(name: str, yb, bus_type):
    """(P, Q, R) of the reference's compiled klu_analyze for grid `name`, as
    tests/golden/make_golden.py stored it (<name>.npz or <name>_order.npz).
    Raises if the fixture belongs to another Y-bus pattern or bus types."""
    path = os.path.join(GOLDEN, f"{name}.npz")
    if not os.path.exists(path):
        path = os.path.join(GOLDEN, f"{name}_order.npz")
    with np.load(path) as z:
        if "pattern_sha256" in z.files:
            same = str(z["pattern_sha256"]) == pattern_fingerprint(yb, bus_type)
        else:
            same = (np.array_equal(z["y_indptr"], yb.indptr)
                    and np.array_equal(z["y_indices"], yb.indices)
                    and np.array_equal(z["bus_type"], bus_type))
        if not same:
            raise ValueError(f"{path}: the fixture's ordering belongs to another pattern")
        return z["ref_P"].copy(), z["ref_Q"].copy(), z["ref_R"].copy()


# ---------------------------------------------------------------------------
# the reference's compiled KLU (only where it was built)

_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_LIB)
        R.ref_analyze.restype = C.c_int
        R.ref_analyze.argtypes = [C.c_int, _i32p, _i32p, _i32p, _i32p, _i32p]
        R.ref_new.restype = C.c_void_p
        R.ref_new.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.POINTER(C.c_int)]
        R.ref_free.argtypes = [C.c_void_p]
        R.ref_sizes.argtypes = [C.c_void_p, _i32p]
        R.ref_symbolic.argtypes = [C.c_void_p, _i32p, _i32p, _i32p]
        R.ref_extract.restype = C.c_int
        R.ref_extract.argtypes = [C.c_void_p] + [_i32p, _i32p, _f64p] * 3 + [_i32p] * 3
        R.ref_refactor_solve.restype = C.c_int
        R.ref_refactor_solve.argtypes = [C.c_void_p, _f64p, _f64p]
        R.ref_refactor.restype = C.c_int
        R.ref_refactor.argtypes = [C.c_void_p, _f64p]
        R.ref_solve.restype = C.c_int
        R.ref_solve.argtypes = [C.c_void_p, _f64p]
        _ref = R
    return _ref


def ref_analyze(n, Ap, Ai):
    """klu_analyze (BTF + AMD, scale 0): returns (P, Q, R)."""
    R = ref()
    P = np.zeros(n, np.int32)
    Q = np.zeros(n, np.int32)
    RR = np.zeros(n + 1, np.int32)
    nb = R.ref_analyze(n, _p(_i32(Ap), _i32p), _p(_i32(Ai), _i32p), _p(P, _i32p), _p(Q, _i32p),
                       _p(RR, _i32p))
    if nb < 0:
        raise RuntimeError(f"klu_analyze failed ({nb})")
    return P, Q, RR[:nb + 1].copy()


class RefKLU:
    """klu_analyze + klu_factor, then klu_refactor/klu_solve, klu_extract."""

    def __init__(self, n, Ap, Ai, Ax):
        self.R = ref()
        self.n = n
        st = C.c_int(0)
        self.h = self.R.ref_new(n, _p(_i32(Ap), _i32p), _p(_i32(Ai), _i32p), _p(_f64(Ax), _f64p),
                                C.byref(st))
        self.status = st.value
        if not self.h:
            raise ZeroDivisionError(f"klu_factor failed (status {st.value})")

    def symbolic(self):
        s = np.zeros(4, np.int32)
        self.R.ref_sizes(self.h, _p(s, _i32p))
        P = np.zeros(self.n, np.int32)
        Q = np.zeros(self.n, np.int32)
        RR = np.zeros(int(s[3]) + 1, np.int32)
        self.R.ref_symbolic(self.h, _p(P, _i32p), _p(Q, _i32p), _p(RR, _i32p))
        return P, Q, RR

    def extract(self):
        s = np.zeros(4, np.int32)
        self.R.ref_sizes(self.h, _p(s, _i32p))
        lnz, unz, nzoff, nb = [int(v) for v in s]
        n = self.n
        out = dict(Lp=np.zeros(n + 1, np.int32), Li=np.zeros(lnz, np.int32), Lx=np.zeros(lnz),
                   Up=np.zeros(n + 1, np.int32), Ui=np.zeros(unz, np.int32), Ux=np.zeros(unz),
                   Fp=np.zeros(n + 1, np.int32), Fi=np.zeros(max(nzoff, 1), np.int32),
                   Fx=np.zeros(max(nzoff, 1)), P=np.zeros(n, np.int32), Q=np.zeros(n, np.int32),
                   R=np.zeros(nb + 1, np.int32))
        ok = self.R.ref_extract(self.h, *[_p(out[k], _i32p if out[k].dtype == np.int32 else _f64p)
                                          for k in ("Lp", "Li", "Lx", "Up", "Ui", "Ux", "Fp",
                                                    "Fi", "Fx", "P", "Q", "R")])
        if not ok:
            raise RuntimeError("klu_extract failed")
        out["Fi"] = out["Fi"][:nzoff]
        out["Fx"] = out["Fx"][:nzoff]
        return out

    def refactor_solve(self, Ax, b):
        x = _f64(b).copy()
        st = self.R.ref_refactor_solve(self.h, _p(_f64(Ax), _f64p), _p(x, _f64p))
        return st, x

    def __del__(self):
        try:
            self.R.ref_free(self.h)
        except Exception:
            pass


def linear_initial_guess(yb, bus_type, p_spec, q_spec, vm, va, zip_imp=None, zip_cur=None):
    """Restatement of the reference's linear_initial_guess
    (src/network.rs:627-678) for one scenario: returns (vm, va) with the PQ
    buses' voltages replaced by the solution of Y'_nn U_n = -Y'_ns U_s, where
    Y' adds y_load = -conj(p + jq) to the diagonal of each PQ bus (:656-657)
    and U_s = from_polar(vm, va) of every other bus moves to the right-hand
    side (:666-669); a bus without a diagonal Y entry gets y_load alone
    (:673-675).  The reference solves the complex system with faer's sparse
    LU (src/sparse.rs:48-63, faer 0.24.4, not vendored); scipy's splu
    stands in for it (results agree to rounding, not bit for bit).  A
    singular or non-finite solve leaves the voltages as they were
    (:677-678, sparse.rs:58-61)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    vm = np.array(vm, dtype=np.float64)
    va = np.array(va, dtype=np.float64)
    n = yb.n
    unknown = [i for i in range(n) if int(bus_type[i]) == 1]
    if not unknown:
        return vm, va
    m = len(unknown)
    pos = -np.ones(n, dtype=np.int64)
    pos[unknown] = np.arange(m)
    rows, cols, vals = [], [], []
    rhs = np.zeros(m, dtype=np.complex128)
    for r, i in enumerate(unknown):
        s_eff = complex(p_spec[i], q_spec[i])  # effective_injection at the bus's |V|
        if zip_imp is not None:
            s_eff += complex(zip_imp[i]) * vm[i] * vm[i]
        if zip_cur is not None:
            s_eff += complex(zip_cur[i]) * vm[i]
        y_load = -np.conj(s_eff)
        diag_seen = False
        for e in range(int(yb.indptr[i]), int(yb.indptr[i + 1])):
            j = int(yb.indices[e])
            y = complex(yb.re[e], yb.im[e])
            if j == i:
                diag_seen = True
                y = y + y_load
            if pos[j] >= 0:
                rows.append(r)
                cols.append(int(pos[j]))
                vals.append(y)
            else:
                rhs[r] -= y * (vm[j] * complex(np.cos(va[j]), np.sin(va[j])))
        if not diag_seen:
            rows.append(r)
            cols.append(r)
            vals.append(y_load)
    a = sp.csc_matrix((np.array(vals), (rows, cols)), shape=(m, m))
    try:
        sol = spla.splu(a).solve(rhs)
    except RuntimeError:
        return vm, va
    if not np.all(np.isfinite(sol)):
        return vm, va
    vm[unknown] = np.abs(sol)
    va[unknown] = np.angle(sol)
    return vm, va
