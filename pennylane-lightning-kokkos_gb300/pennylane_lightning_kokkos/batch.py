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

    _OP_DTYPE = np.dtype([("gate", "<i4"), ("nw", "<i4"), ("adj", "<i4"), ("np", "<i4"), ("w", "<u8"), ("p", "<u8"),
                          ("m", "<u8")])

    def add(self, num_qubits: int, ops: Sequence, observable: Sequence, trainable: Sequence[int] | None = None) -> int:
        """Adds a circuit given as an op list; returns its index."""
        wl = [op[1] for op in ops]
        pl = [op[3] if len(op) > 3 else () for op in ops]
        pk = {"gates": np.array([N.GATE_ID[op[0]] for op in ops], dtype=np.int32),
              "wire_offsets": np.concatenate([[0], np.cumsum([len(w) for w in wl])]).astype(np.int64),
              "wires": np.array([int(x) for w in wl for x in w], dtype=np.int64),
              "inverse": np.array([bool(op[2]) if len(op) > 2 else False for op in ops], dtype=np.int32),
              "param_offsets": np.concatenate([[0], np.cumsum([len(p) for p in pl])]).astype(np.int64),
              "params": np.array([float(x) for p in pl for x in p], dtype=np.float64),
              "matrices": {i: op[4] for i, op in enumerate(ops) if op[0] == "Matrix"}}
        return self.add_packed(num_qubits, pk, observable, trainable)

    def add_packed(self, num_qubits: int, pk: dict, observable: Sequence, trainable: Sequence[int] | None = None) -> int:
        """Adds a circuit given as flat arrays (see circuits.layered_ansatz_arrays)."""
        gates = np.ascontiguousarray(pk["gates"], dtype=np.int32)
        nops = len(gates)
        wo = np.asarray(pk["wire_offsets"], dtype=np.int64)
        po = np.asarray(pk["param_offsets"], dtype=np.int64)
        wires_all = np.ascontiguousarray(pk["wires"], dtype=np.int64)
        params_all = np.ascontiguousarray(pk["params"], dtype=np.float64)
        if len(wires_all) == 0:
            wires_all = np.zeros(1, dtype=np.int64)
        if len(params_all) == 0:
            params_all = np.zeros(1, dtype=np.float64)
        keep = [wires_all, params_all]
        arr = np.zeros(max(1, nops), dtype=self._OP_DTYPE)
        if nops:
            npar = np.diff(po)
            arr["gate"][:nops] = gates
            arr["nw"][:nops] = np.diff(wo)
            arr["adj"][:nops] = np.asarray(pk["inverse"], dtype=np.int32)
            arr["np"][:nops] = npar
            arr["w"][:nops] = wires_all.ctypes.data + 8 * wo[:-1].astype(np.uint64)
            arr["p"][:nops] = np.where(npar > 0, params_all.ctypes.data + 8 * po[:-1].astype(np.uint64), 0)
            for i, m in pk.get("matrices", {}).items():
                mm = np.ascontiguousarray(np.asarray(m, dtype=np.complex128))
                keep.append(mm)
                arr["m"][i] = mm.ctypes.data
        coeffs = np.ascontiguousarray([float(c) for c, _, _ in observable], dtype=np.float64)
        offs = np.ascontiguousarray(np.cumsum([0] + [len(w) for _, w, _ in observable]), dtype=np.int64)
        wires = np.ascontiguousarray([x for _, w, _ in observable for x in w] or [0], dtype=np.int64)
        letters = "".join(l for _, _, l in observable).encode()
        tp = None if trainable is None else np.ascontiguousarray(trainable, dtype=np.int64)
        idx = C.c_int64()
        N.check(N.lib.plk_batch_add(self._h, num_qubits, C.cast(arr.ctypes.data, C.POINTER(N.PlkOp)), nops,
                                    _p(tp, _i64p) if tp is not None else None, 0 if tp is None else len(tp),
                                    len(coeffs), _p(coeffs, _dp), _p(offs, _i64p), _p(wires, _i64p), letters,
                                    C.byref(idx)))
        del keep
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

    def set_config(self, cluster=8, threads=256, smem_qubits=None, cluster_min_qubits=17, ctas_per_sm=1):
        N.check(N.lib.plk_batch_set_occupancy(self._h, ctas_per_sm))
        if smem_qubits is None:
            smem_qubits = 13 if self.dtype == "c64" and ctas_per_sm == 1 else 12
        N.check(N.lib.plk_batch_set_config(self._h, cluster, threads, smem_qubits, cluster_min_qubits))

    def get_config(self):
        v = [C.c_int32() for _ in range(5)]
        N.check(N.lib.plk_batch_get_config(self._h, *[C.byref(x) for x in v[:4]]))
        N.check(N.lib.plk_batch_get_occupancy(self._h, C.byref(v[4])))
        return dict(zip(("cluster", "threads", "smem_qubits", "cluster_min_qubits", "ctas_per_sm"),
                        [x.value for x in v]))

    def set_graph(self, use: bool) -> None:
        N.check(N.lib.plk_batch_set_graph(self._h, int(use)))

    def tune(self, reps: int = 3) -> str:
        buf = C.create_string_buffer(8192)
        N.check(N.lib.plk_batch_tune(self._h, reps, buf, len(buf)))
        return buf.value.decode()


# --------------------------------------------------------------- sharding --
def shard_plan(costs: Sequence[float], world: int) -> list:
    """Cost-balanced assignment of independent circuits to `world` GPUs:
    circuits in decreasing cost (ties: lower index first), each to the GPU
    with the least work so far (ties: lower rank).  `costs` are per-circuit
    work estimates, e.g. gates x 2^qubits.  Returns, per rank, the circuit
    indices it runs, in increasing order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    shards = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        shards[r].append(i)
        load[r] += float(costs[i])
    return [sorted(s) for s in shards]


def gather_shards(dist, shards: list, expvals, grads, root: int = 0):
    """Reassembles per-rank results in circuit order on `root`: each rank
    passes the expectation values and gradient arrays of its own shard (in
    the shard's order).  The results travel once, as host objects, at the end
    of a run (the circuits themselves need no exchange).  Returns
    (expvals, grads) over all circuits on `root`, (None, None) elsewhere."""
    rank = dist.get_rank()
    payload = (list(map(float, expvals)), [np.asarray(g, dtype=np.float64) for g in grads])
    gathered = [None] * dist.get_world_size() if rank == root else None
    dist.gather_object(payload, gathered, dst=root)
    if rank != root:
        return None, None
    n = sum(len(s) for s in shards)
    ev_all, g_all = [None] * n, [None] * n
    for r, (ev_r, g_r) in enumerate(gathered):
        if len(ev_r) != len(shards[r]) or len(g_r) != len(shards[r]):
            raise RuntimeError(f"rank {r} returned {len(ev_r)} results for a shard of {len(shards[r])} circuits")
        for k, i in enumerate(shards[r]):
            ev_all[i], g_all[i] = ev_r[k], g_r[k]
    return np.array(ev_all), g_all


def run_shard(workload: Sequence, shard: Sequence[int], dtype: str = "c64", device: int = 0):
    """Runs this rank's circuits of `workload` ([(num_qubits, packed ops,
    words)], as circuits.batch_workload_packed) in one CircuitBatch; returns
    (expvals, gradients) in the shard's order."""
    b = CircuitBatch(dtype, device)
    try:
        for i in shard:
            nq, pk, words = workload[i]
            b.add_packed(nq, pk, words)
        ev, jac = b.run()
        return ev, b.gradients(jac)
    finally:
        b.close()
