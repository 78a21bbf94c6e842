"""Test-side access to the oracles (test infrastructure only).

* ``run_oracle``: the CPU restatement in oracle/sigma_oracle.cpp, loaded with ctypes
  from oracle/_build/libsigma_oracle.so (built by ``__graft_entry__.build()``).
* ``run_reference``: the compiled reference harness oracle/_ref/sigma_ref (built from
  the reference sources by oracle/ref.mk; only present where the reference is).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

from parafrost_gb300 import cnfgen, rounddump
from parafrost_gb300.options import Options

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "libsigma_oracle.so")
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "sigma_ref")
REF_SOLVER = os.path.join(ROOT, "oracle", "_ref", "parafrost")

_lib = None


def oracle_lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            raise RuntimeError(f"oracle library missing: {ORACLE_SO} (run __graft_entry__.build())")
        _lib = ctypes.CDLL(ORACLE_SO)
        _lib.oracle_sigmify.restype = ctypes.c_int
        _lib.oracle_sigmify.argtypes = [
            ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
            ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        _lib.oracle_check_drat.restype = ctypes.c_long
        _lib.oracle_check_drat.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                           ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(ctypes.c_int)]
        _lib.oracle_extend_and_check.restype = ctypes.c_long
        _lib.oracle_extend_and_check.argtypes = [ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
    return _lib


def check_models(num_vars, lits, offsets, status, res, model) -> list:
    """Properties of a simplified formula for a model of the original (uint8 per
    variable, 1 = true): every surviving clause and every unit holds under it (they
    are all implied by the original), and the model restricted to the variables that
    were not eliminated, extended through the witness stack as MODEL::extend does,
    satisfies every original clause. Returns the failures found (empty = none)."""
    fails = []
    if status != 0:
        return ["round reported UNSAT for a satisfiable formula"]
    model = np.ascontiguousarray(model, dtype=np.uint8)
    truth = model[res.lits >> 1] == (1 - (res.lits & 1)).astype(np.uint8)
    o = res.offsets.astype(np.int64)
    if o.size > 1:
        nonempty = o[1:] > o[:-1]
        if not nonempty.all():
            fails.append("empty clause in the result")
        sat = np.logical_or.reduceat(truth, o[:-1][nonempty]) if truth.size else np.zeros(0, bool)
        if not sat.all():
            fails.append(f"{int((~sat).sum())} result clauses false under the original's model")
    u = res.units
    if u.size and not (model[u >> 1] == (1 - (u & 1))).all():
        fails.append("a unit is false under the original's model")
    v = model.copy()
    v[np.asarray(res.eliminated, dtype=bool)] = 0
    lits = np.ascontiguousarray(lits, dtype=np.uint32)
    offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
    resolved = np.ascontiguousarray(res.resolved, dtype=np.uint32)
    bad = oracle_lib().oracle_extend_and_check(num_vars, v.ctypes.data, resolved.ctypes.data, resolved.size,
                                               lits.ctypes.data, offsets.ctypes.data, offsets.size - 1)
    if bad != 0:
        fails.append(f"extended model falsifies {bad} original clauses" if bad > 0 else "malformed witness stack")
    return fails


def run_oracle(num_vars, lits, offsets, opts: Options | None = None, level: int = 2, learnt=None):
    """Run the restated round; returns (status, records, seconds)."""
    opts = opts or Options(all=1)
    o = opts.derived().to_struct()
    lits = np.ascontiguousarray(lits, dtype=np.uint32)
    offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
    lp = None
    if learnt is not None:
        learnt = np.ascontiguousarray(learnt, dtype=np.uint8)
        lp = learnt.ctypes.data
    secs = ctypes.c_double(0.0)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "oracle.dump")
        st = oracle_lib().oracle_sigmify(ctypes.addressof(o), num_vars, lits.ctypes.data, offsets.ctypes.data,
                                         offsets.size - 1, lp, path.encode(), level, ctypes.byref(secs))
        recs = rounddump.read(path)
    return st, recs, secs.value


def reference_available() -> bool:
    return os.path.exists(REF_BIN)


def run_reference(num_vars, lits, offsets, opts: Options | None = None, level: int = 2, learnt_tail: int = 0,
                  proof: bool = False):
    """Run the compiled reference round through its own DIMACS parser; returns records
    (with proof, (records, the round's binary DRAT lines)). With learnt_tail, the last
    learnt_tail clauses enter the round as learnt clauses."""
    opts = opts or Options(all=1)
    with tempfile.TemporaryDirectory() as td:
        cnf = os.path.join(td, "f.cnf")
        dump = os.path.join(td, "ref.dump")
        prf = os.path.join(td, "ref.proof")
        cnfgen.to_dimacs(cnf, num_vars, lits, offsets)
        args = [REF_BIN, cnf, dump, str(level)] + ([f"--learnt-tail={learnt_tail}"] if learnt_tail else [])
        args += opts.reference_flags() + (["-proof", f"--proofout={prf}"] if proof else [])
        subprocess.run(args, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        recs = rounddump.read(dump)
        if not proof:
            return recs
        with open(prf, "rb") as f:
            lines = drat_lines(f.read())
        mark = [d for (k, ph, st, d) in recs if k == "proofmark"]
        return recs, lines[int(mark[0][0]) if mark else 0:]


def solver_available() -> bool:
    return os.path.exists(REF_SOLVER)


def reference_solve(num_vars, lits, offsets, units=(), timeout: float = 600.0):
    """Solve a formula (plus unit clauses) with the compiled reference CDCL solver,
    its own simplifier off (-no-sigma -no-sigmalive). Returns ("SAT", model) with
    model a uint8 array over variables 0..num_vars (1 = true), or ("UNSAT", None)."""
    lits = np.ascontiguousarray(lits, dtype=np.uint32)
    offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
    units = np.asarray(units, dtype=np.uint32)
    if units.size:
        lits = np.concatenate([lits[int(offsets[0]):int(offsets[-1])], units])
        offsets = np.concatenate([offsets - offsets[0], offsets[-1] - offsets[0] + 1 + np.arange(units.size, dtype=np.uint64)])
    with tempfile.TemporaryDirectory() as td:
        cnf = os.path.join(td, "f.cnf")
        cnfgen.to_dimacs(cnf, num_vars, lits, offsets)
        out = subprocess.run([REF_SOLVER, cnf, "-quiet", "-no-sigma", "-no-sigmalive", "-model", "-modelprint"],
                             check=True, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
                             timeout=timeout).stdout
    status = [l.split()[1] for l in out.splitlines() if l.startswith("s ")]
    if status == ["UNSATISFIABLE"]:
        return "UNSAT", None
    if status != ["SATISFIABLE"]:
        raise RuntimeError(f"reference solver answered {status}")
    model = np.zeros(num_vars + 1, dtype=np.uint8)
    for line in out.splitlines():
        if line.startswith("v "):
            for tok in line.split()[1:]:
                x = int(tok)
                if x > 0:
                    model[x] = 1
    return "SAT", model


def check_drat(num_vars, lits, offsets, proof: bytes):
    """(first failing line or -1 when every addition is RUP, refutes) of a binary DRAT
    proof against the formula (-2: malformed)."""
    lits = np.ascontiguousarray(lits, dtype=np.uint32)
    offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
    buf = np.frombuffer(proof, dtype=np.uint8) if len(proof) else np.zeros(1, np.uint8)
    empty = ctypes.c_int(0)
    r = oracle_lib().oracle_check_drat(num_vars, lits.ctypes.data, offsets.ctypes.data, offsets.size - 1,
                                       buf.ctypes.data, len(proof), ctypes.byref(empty))
    return int(r), bool(empty.value)


def drat_lines(proof: bytes) -> list:
    """[(tag, (lit, ...))] of a binary DRAT proof."""
    out, p, n = [], 0, len(proof)
    while p < n:
        tag = chr(proof[p])
        p += 1
        lits = []
        while True:
            r, shift = 0, 0
            while True:
                b = proof[p]
                p += 1
                r |= (b & 127) << shift
                shift += 7
                if not b & 128:
                    break
            if r == 0:
                break
            lits.append(r)
        out.append((tag, tuple(lits)))
    return out
