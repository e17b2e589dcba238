"""Batches of independent circuits: forward, <H> and adjoint gradient together.

``CircuitBatch`` collects circuits, each with its own qubit count, gate list,
parameters and Pauli-sum observable, and evaluates all of them in one
persistent GPU launch replayed as a CUDA graph (``plk_batch_*`` in the C ABI).
For every circuit it returns what the reference device computes per tape:
the expectation value of the observable after the circuit
(``LightningKokkos.expval``, lightning_kokkos.py:403-430) and its adjoint
Jacobian over the trainable parameters
(``LightningKokkos.adjoint_jacobian``, lightning_kokkos.py:623-687).

Ops are ``(name, wires)``, ``(name, wires, inverse)``,
``(name, wires, inverse, params)`` or ``(name, wires, inverse, params,
matrix)`` for ``name == "Matrix"``; gates act on at most four wires (MultiRZ
on any number).  A circuit's parameters form a flat list in op order (Rot and
CRot contribute three, all differentiable).  Observables are
``[(coeff, wires, letters)]`` Pauli words, e.g. ``(0.5, [0, 3], "XZ")``.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _native as N

_i64p, _dp = C.POINTER(C.c_int64), C.POINTER(C.c_double)


def _p(a, t):
    return a.ctypes.data_as(t)


class CircuitBatch:
    def __init__(self, dtype: str = "c64", device: int = 0):
        if dtype not in ("c64", "c128"):
            raise ValueError("dtype must be 'c64' or 'c128'")
        self.dtype = dtype
        self._h = C.c_void_p()
        N.check(N.lib.plk_batch_create(N.PLK_C64 if dtype == "c64" else N.PLK_C128, device, C.byref(self._h)))
        self.num_circuits = 0

    def close(self):
        if getattr(self, "_h", None):
            N.lib.plk_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def add(self, num_qubits: int, ops: Sequence, observable: Sequence, trainable: Sequence[int] | None = None) -> int:
        keep = []
        arr = (N.PlkOp * max(1, len(ops)))()
        for i, op in enumerate(ops):
            name, wires = op[0], op[1]
            inv = bool(op[2]) if len(op) > 2 else False
            prm = np.ascontiguousarray(np.asarray(op[3] if len(op) > 3 else [], dtype=np.float64).reshape(-1))
            w = np.ascontiguousarray(np.asarray(wires, dtype=np.int64).reshape(-1))
            mat = None
            if name == "Matrix":
                m = np.ascontiguousarray(np.asarray(op[4], dtype=np.complex128))
                mat = m.view(np.float64)
                keep.append(mat)
            keep += [prm, w]
            arr[i] = N.PlkOp(N.GATE_ID[name], len(w), int(inv), len(prm), _p(w, _i64p),
                             _p(prm, _dp) if len(prm) else None, _p(mat, _dp) if mat is not None else None)
        coeffs = np.ascontiguousarray([float(c) for c, _, _ in observable], dtype=np.float64)
        offs = np.ascontiguousarray(np.cumsum([0] + [len(w) for _, w, _ in observable]), dtype=np.int64)
        wires = np.ascontiguousarray([x for _, w, _ in observable for x in w] or [0], dtype=np.int64)
        letters = "".join(l for _, _, l in observable).encode()
        tp = None if trainable is None else np.ascontiguousarray(trainable, dtype=np.int64)
        idx = C.c_int64()
        N.check(N.lib.plk_batch_add(self._h, num_qubits, arr, len(ops), _p(tp, _i64p) if tp is not None else None,
                                    0 if tp is None else len(tp), len(coeffs), _p(coeffs, _dp), _p(offs, _i64p),
                                    _p(wires, _i64p), letters, C.byref(idx)))
        self.num_circuits += 1
        return idx.value

    def info(self):
        nc, npar, nj = C.c_int64(), C.c_int64(), C.c_int64()
        N.check(N.lib.plk_batch_info(self._h, C.byref(nc), C.byref(npar), C.byref(nj)))
        return nc.value, npar.value, nj.value

    def circuit_info(self, c: int):
        po, npar, jo, ntp = C.c_int64(), C.c_int32(), C.c_int64(), C.c_int32()
        N.check(N.lib.plk_batch_circuit_info(self._h, c, C.byref(po), C.byref(npar), C.byref(jo), C.byref(ntp)))
        return po.value, npar.value, jo.value, ntp.value

    def set_params(self, params) -> None:
        p = np.ascontiguousarray(params, dtype=np.float64).reshape(-1)
        N.check(N.lib.plk_batch_set_params(self._h, _p(p, _dp), len(p)))

    def run(self, params=None):
        """Returns (expvals [num_circuits], flat Jacobian [sum of trainables])."""
        if params is not None:
            self.set_params(params)
        nc, _, nj = self.info()
        ev = np.zeros(nc)
        jac = np.zeros(max(nj, 1))
        N.check(N.lib.plk_batch_run(self._h, _p(ev, _dp), _p(jac, _dp)))
        return ev, jac[:nj]

    def gradients(self, jac):
        """Splits a flat Jacobian into one array per circuit."""
        out = []
        for c in range(self.num_circuits):
            _, _, jo, ntp = self.circuit_info(c)
            out.append(jac[jo:jo + ntp])
        return out

    def last_time(self):
        ms, n = C.c_double(), C.c_int64()
        N.check(N.lib.plk_batch_last_time(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def set_config(self, cluster=8, threads=256, smem_qubits=None, cluster_min_qubits=17):
        if smem_qubits is None:
            smem_qubits = 13 if self.dtype == "c64" else 12
        N.check(N.lib.plk_batch_set_config(self._h, cluster, threads, smem_qubits, cluster_min_qubits))

    def get_config(self):
        v = [C.c_int32() for _ in range(4)]
        N.check(N.lib.plk_batch_get_config(self._h, *[C.byref(x) for x in v]))
        return dict(zip(("cluster", "threads", "smem_qubits", "cluster_min_qubits"), [x.value for x in v]))

    def set_graph(self, use: bool) -> None:
        N.check(N.lib.plk_batch_set_graph(self._h, int(use)))

    def tune(self, reps: int = 3) -> str:
        buf = C.create_string_buffer(8192)
        N.check(N.lib.plk_batch_tune(self._h, reps, buf, len(buf)))
        return buf.value.decode()
