"""Test-side helpers that drive the GB300 core through its C ABI (ctypes).

The parity tests call the kernels exactly as a foreign caller would: plain
pointers and sizes into ``libplk_gb300.so``; states come back as numpy arrays
and are compared with the oracle.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from pennylane_lightning_kokkos import _native as N

CDT = {N.PLK_C64: np.complex64, N.PLK_C128: np.complex128}


def i64(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.int64).reshape(-1))
    return a, a.ctypes.data_as(C.POINTER(C.c_int64))


def f64(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def cmat(m):
    """complex matrix -> interleaved complex128 buffer"""
    a = np.ascontiguousarray(np.asarray(m, dtype=np.complex128).reshape(-1))
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


class State:
    def __init__(self, nq, dtype=N.PLK_C128, device=0):
        self.nq, self.dtype = nq, dtype
        h = C.c_void_p()
        N.check(N.lib.plk_state_create(nq, dtype, device, C.byref(h)))
        self.h = h

    @classmethod
    def from_array(cls, arr, dtype=N.PLK_C128):
        arr = np.asarray(arr)
        nq = int(arr.size).bit_length() - 1
        s = cls(nq, dtype)
        s.set(arr)
        return s

    def close(self):
        if self.h:
            N.lib.plk_state_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set(self, arr):
        a = np.ascontiguousarray(np.asarray(arr, dtype=CDT[self.dtype]))
        assert a.size == 1 << self.nq
        N.check(N.lib.plk_state_h2d(self.h, a.ctypes.data_as(C.c_void_p), a.size))
        return self

    def get(self):
        out = np.empty(1 << self.nq, dtype=CDT[self.dtype])
        N.check(N.lib.plk_state_d2h(self.h, out.ctypes.data_as(C.c_void_p), out.size))
        return out

    def apply(self, name, wires, inverse=False, params=()):
        w, wp = i64(wires)
        p, pp = f64(params if len(params) else [0.0])
        N.check(N.lib.plk_apply_gate(self.h, N.GATE_ID[name], wp, len(w), int(bool(inverse)), pp, len(params)))
        return self

    def apply_matrix(self, m, wires, inverse=False):
        mm, mp = cmat(m)
        w, wp = i64(wires)
        N.check(N.lib.plk_apply_matrix(self.h, mp, wp, len(w), int(bool(inverse))))
        return self

    def generator(self, name, wires):
        w, wp = i64(wires)
        s = C.c_double()
        N.check(N.lib.plk_apply_generator(self.h, N.GATE_ID[name], wp, len(w), 0, C.byref(s)))
        return s.value

    def expval_named(self, name, wires):
        w, wp = i64(wires)
        out = C.c_double()
        N.check(N.lib.plk_expval_named(self.h, N.GATE_ID[name], wp, len(w), C.byref(out)))
        return out.value

    def expval_matrix(self, m, wires):
        mm, mp = cmat(m)
        w, wp = i64(wires)
        out = C.c_double()
        N.check(N.lib.plk_expval_matrix(self.h, mp, wp, len(w), C.byref(out)))
        return out.value

    def probs(self, wires=()):
        w, wp = i64(wires if len(wires) else [0])
        out = np.empty(1 << (len(wires) if len(wires) else self.nq), dtype=np.float64)
        N.check(N.lib.plk_probs(self.h, wp, len(wires), out.ctypes.data_as(C.POINTER(C.c_double))))
        return out


def make_ops(ops):
    """[(name, wires, inverse, params[, matrix])] -> (PlkOp array, keepalive)"""
    keep = []
    arr = (N.PlkOp * max(1, len(ops)))()
    for i, op in enumerate(ops):
        name, wires, inv, params = op[:4]
        w, wp = i64(wires)
        p, pp = f64(params if len(params) else [0.0])
        keep += [w, p]
        mptr = None
        gate = N.GATE_ID[name] if name in N.GATE_ID else N.GATE_MATRIX
        if len(op) > 4 and op[4] is not None:
            m, mptr = cmat(op[4])
            keep.append(m)
            gate = N.GATE_MATRIX
        arr[i] = N.PlkOp(gate, len(w), int(bool(inv)), len(params), wp, pp, mptr)
    return arr, keep
