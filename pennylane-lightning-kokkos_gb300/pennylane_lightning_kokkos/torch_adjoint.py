"""Expectation values of parametrised circuits as a differentiable torch op.

``AdjointCircuit(num_qubits, ops, observables)`` is a callable whose forward
runs the circuit on the GPU through the C ABI and returns ``<H_j>`` for each
Pauli-sum observable, and whose backward is the adjoint method: one fused
backward sweep (``plk_adjoint_jacobian``) for the vector-Jacobian product,
with the incoming gradient folded into a single observable sum_j g_j H_j (the
same trick as the reference's ``LightningKokkos.vjp``, lightning_kokkos.py:
689-728).

Memory: the backward sweep needs the forward state lambda, a working copy and
H lambda.  When three states do not fit in free device memory (or
``recompute=True``), the forward state is not kept: backward re-runs the
forward pass and sweeps in place (``plk_adjoint_jacobian_inplace``), so two
states suffice.

Precision: ``dtype="c64"`` stores the state in complex64 (half the bytes per
sweep) while expectation values and gradient inner products accumulate in
FP64-class arithmetic; ``dtype="c128"`` stores complex128.  Gradients are
returned as float64.

Only single-parameter gates are differentiable (as in the reference, which
rejects multi-parameter ops, AdjointDiffKokkos.hpp:444-446); ``Rot`` is
decomposed into RZ, RY, RZ like the reference's serializer does
(_serialize.py:283-284).
"""
from __future__ import annotations

import ctypes as C
from typing import Iterable, Sequence

import numpy as np
import torch

from . import _native as N

PAULI = {"X", "Y", "Z", "I"}


class PauliSum:
    """sum_t c_t P_t with P_t a product of Pauli letters on distinct wires."""

    def __init__(self, words: Iterable):
        self.words = [(float(c), [int(w) for w in wires], str(letters)) for c, wires, letters in words]
        for c, wires, letters in self.words:
            if len(wires) != len(letters) or any(l not in PAULI for l in letters):
                raise ValueError(f"bad Pauli word {letters} on {wires}")

    def packed(self, scale: float = 1.0):
        coeffs = np.array([c * scale for c, _, _ in self.words], dtype=np.float64)
        offs = np.cumsum([0] + [len(w) for _, w, _ in self.words]).astype(np.int64)
        wires = np.array([x for _, w, _ in self.words for x in w] or [0], dtype=np.int64)
        letters = "".join(l for _, _, l in self.words).encode()
        return coeffs, offs, wires, letters


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class _State:
    def __init__(self, nq, dtype, device, stream):
        self.h = C.c_void_p()
        N.check(N.lib.plk_state_create(nq, dtype, device, C.byref(self.h)))
        N.check(N.lib.plk_state_set_stream(self.h, C.c_void_p(stream)))

    def free(self):
        if self.h:
            N.lib.plk_state_destroy(self.h)
            self.h = None

    __del__ = free


class AdjointCircuit:
    """Differentiable <H_j>(params) of a fixed circuit structure.

    ops: [(name, wires)] or [(name, wires, inverse)]; every parametric op
    consumes the next entry of the parameter vector (Rot consumes three and is
    decomposed).  observables: PauliSum or [(coeff, wires, letters)] lists.
    """

    def __init__(self, num_qubits: int, ops: Sequence, observables: Sequence, dtype: str = "c64", device: int = 0,
                 recompute="auto"):
        if dtype not in ("c64", "c128"):
            raise ValueError("dtype must be 'c64' or 'c128'")
        self.nq, self.device, self.recompute = int(num_qubits), int(device), recompute
        self.dtype = N.PLK_C64 if dtype == "c64" else N.PLK_C128
        self.observables = [o if isinstance(o, PauliSum) else PauliSum(o) for o in observables]
        # expand to single-parameter ops; remember which parameter each op reads
        self.ops = []  # (gate id, wires, inverse, param index or -1)
        k = 0
        for op in ops:
            name, wires = op[0], [int(w) for w in op[1]]
            inv = bool(op[2]) if len(op) > 2 else False
            if name == "Rot":
                if inv:
                    raise ValueError("inverse Rot is not supported; invert its decomposition instead")
                for sub in ("RZ", "RY", "RZ"):
                    self.ops.append((N.GATE_ID[sub], wires, False, k))
                    k += 1
                continue
            if name not in N.GATE_ID or name == "Matrix":
                raise ValueError(f"unknown gate {name}")
            g = N.GATE_ID[name]
            npar = N.lib.plk_gate_num_params(g)
            if npar > 1:
                raise ValueError(f"{name} has {npar} parameters; only single-parameter gates are differentiable")
            self.ops.append((g, wires, inv, k if npar == 1 else -1))
            k += npar
        self.num_params = k
        self._wire_arrays = [np.array(w, dtype=np.int64) for _, w, _, _ in self.ops]

    # -- helpers -----------------------------------------------------------
    def _tape(self, params: np.ndarray):
        arr = (N.PlkOp * max(1, len(self.ops)))()
        keep = []
        for i, (g, _, inv, pi) in enumerate(self.ops):
            w = self._wire_arrays[i]
            p = np.array([params[pi] if pi >= 0 else 0.0], dtype=np.float64)
            keep.append(p)
            arr[i] = N.PlkOp(g, len(w), int(inv), 1 if pi >= 0 else 0, _ptr(w, C.c_int64), _ptr(p, C.c_double), None)
        return arr, keep

    def _stream(self):
        return torch.cuda.current_stream(self.device).cuda_stream

    def _run_forward(self, params: np.ndarray) -> _State:
        st = _State(self.nq, self.dtype, self.device, self._stream())
        arr, keep = self._tape(params)
        N.check(N.lib.plk_apply_ops(st.h, arr, len(self.ops)))
        return st

    def _expvals(self, st: _State) -> np.ndarray:
        out = np.zeros(len(self.observables))
        v = C.c_double()
        for j, obs in enumerate(self.observables):
            c, o, w, l = obs.packed()
            N.check(N.lib.plk_expval_pauli_sum(st.h, len(c), _ptr(c, C.c_double), _ptr(o, C.c_int64),
                                               _ptr(w, C.c_int64), l, C.byref(v)))
            out[j] = v.value
        return out

    def state_bytes(self) -> int:
        return (1 << self.nq) * (8 if self.dtype == N.PLK_C64 else 16)

    def keeps_forward_state(self) -> bool:
        if self.recompute is True:
            return False
        if self.recompute is False:
            return True
        free, _ = torch.cuda.mem_get_info(self.device)
        return 3 * self.state_bytes() < 0.9 * free

    def vjp(self, params: np.ndarray, grad_out: np.ndarray, state: _State | None) -> np.ndarray:
        """sum_j grad_out[j] d<H_j>/dparams via one adjoint sweep."""
        if self.num_params == 0:
            return np.zeros(0)
        words = [(c * float(g), w, l) for g, obs in zip(grad_out, self.observables) for c, w, l in obs.words]
        hsum = PauliSum(words)
        inplace = state is None
        lam = self._run_forward(params) if inplace else state
        hl = _State(self.nq, self.dtype, self.device, self._stream())
        try:
            c, o, w, l = hsum.packed()
            N.check(N.lib.plk_apply_pauli_sum(hl.h, lam.h, len(c), _ptr(c, C.c_double), _ptr(o, C.c_int64),
                                              _ptr(w, C.c_int64), l))
            arr, keep = self._tape(params)
            tp_ops = [i for i, op in enumerate(self.ops) if op[3] >= 0]
            tp = np.arange(len(tp_ops), dtype=np.int64)
            jac = np.zeros(len(tp_ops))
            harr = (C.c_void_p * 1)(hl.h.value)
            fn = N.lib.plk_adjoint_jacobian_inplace if inplace else N.lib.plk_adjoint_jacobian
            N.check(fn(lam.h, harr, 1, arr, len(self.ops), _ptr(tp, C.c_int64), len(tp), _ptr(jac, C.c_double)))
        finally:
            hl.free()
            if inplace:
                lam.free()
        grad = np.zeros(self.num_params)
        for t, i in enumerate(tp_ops):
            grad[self.ops[i][3]] += jac[t]
        return grad

    def __call__(self, params: torch.Tensor) -> torch.Tensor:
        return _AdjointExpval.apply(params, self)


class _AdjointExpval(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, circuit: AdjointCircuit):
        p = params.detach().to("cpu", torch.float64).numpy().reshape(-1)
        if p.size != circuit.num_params:
            raise ValueError(f"expected {circuit.num_params} parameters, got {p.size}")
        st = circuit._run_forward(p)
        vals = circuit._expvals(st)
        keep = circuit.keeps_forward_state()
        if not keep:
            st.free()
            st = None
        ctx.circuit, ctx.params, ctx.state = circuit, p, st
        ctx.out_device, ctx.out_dtype = params.device, params.dtype
        return torch.as_tensor(vals, dtype=torch.float64, device=params.device)

    @staticmethod
    def backward(ctx, grad_out):
        g = grad_out.detach().to("cpu", torch.float64).numpy().reshape(-1)
        grad = ctx.circuit.vjp(ctx.params, g, ctx.state)
        if ctx.state is not None:
            ctx.state.free()
            ctx.state = None
        return torch.as_tensor(grad, dtype=ctx.out_dtype, device=ctx.out_device), None
