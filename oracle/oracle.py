"""ctypes front end of the CPU oracle (``oracle/plk_oracle.c``).

TEST INFRASTRUCTURE ONLY.  The oracle restates the reference's Kokkos
functors in plain C; ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it as the
checker and as the timed CPU baseline.  The product never imports it.

States are numpy ``complex128`` arrays (the C ``orc_cplx`` layout), wire 0 is
the most significant bit of the amplitude index.

Observables are described with small tuples so that tests can build the same
observable for the oracle and for the product:

    ("named", name, wires)
    ("hermitian", matrix, wires)
    ("tensor", [obs, ...])
    ("hamiltonian", coeffs, [obs, ...])
    ("sparse", data, indices, indptr, wires)

``apply_observable`` follows ``ObservablesKokkos.hpp`` (applyInPlace of each
class: NamedObs :116-118, HermitianObs :172-179, TensorProdObs :272-276,
Hamiltonian :360-373, SparseHamiltonian :484-494).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libplk_oracle.so")
_lock = threading.Lock()
_lib = None


class OracleError(RuntimeError):
    pass


class _Cplx(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def build() -> str:
    """Compile the oracle library (gcc, a few seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                os.path.join(_HERE, "plk_oracle.c")
            ):
                build()
            L = C.CDLL(_LIB_PATH)
            vp, i64p, dp = C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_double)
            L.orc_apply.argtypes = [vp, C.c_int, C.c_char_p, i64p, C.c_int, C.c_int, dp, C.c_int]
            L.orc_apply.restype = C.c_int
            L.orc_apply_matrix.argtypes = [vp, C.c_int, vp, i64p, C.c_int, C.c_int]
            L.orc_apply_matrix.restype = C.c_int
            L.orc_apply_matrix_refmap.argtypes = [vp, C.c_int, vp, i64p, C.c_int, C.c_int]
            L.orc_apply_matrix_refmap.restype = C.c_int
            L.orc_apply_generator.argtypes = [vp, C.c_int, C.c_char_p, i64p, C.c_int, C.c_int,
                                              C.POINTER(C.c_int)]
            L.orc_apply_generator.restype = C.c_double
            L.orc_expval_named.argtypes = [vp, C.c_int, C.c_char_p, i64p, C.c_int, C.POINTER(C.c_int)]
            L.orc_expval_named.restype = C.c_double
            L.orc_expval_matrix.argtypes = [vp, C.c_int, vp, i64p, C.c_int, C.POINTER(C.c_int)]
            L.orc_expval_matrix.restype = C.c_double
            L.orc_expval_sparse.argtypes = [vp, C.c_int64, vp, i64p, i64p]
            L.orc_expval_sparse.restype = C.c_double
            L.orc_axpy.argtypes = [_Cplx, vp, vp, C.c_size_t]
            L.orc_axpy.restype = None
            L.orc_spmv.argtypes = [vp, vp, C.c_int64, vp, i64p, i64p]
            L.orc_spmv.restype = None
            L.orc_inner_re.argtypes = [vp, vp, C.c_size_t]
            L.orc_inner_re.restype = C.c_double
            L.orc_inner_im.argtypes = [vp, vp, C.c_size_t]
            L.orc_inner_im.restype = C.c_double
            L.orc_probs.argtypes = [vp, C.c_int, dp]
            L.orc_probs.restype = None
            L.orc_probs_wires.argtypes = [vp, C.c_int, i64p, C.c_int, dp]
            L.orc_probs_wires.restype = C.c_int
            L.orc_cdf_exclusive.argtypes = [dp, C.c_size_t, dp]
            L.orc_cdf_exclusive.restype = None
            L.orc_sample_from_uniforms.argtypes = [dp, C.c_size_t, C.c_int, dp, C.c_size_t, i64p]
            L.orc_sample_from_uniforms.restype = None
            L.orc_adjoint_jacobian.argtypes = [vp, C.c_int, C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                               C.POINTER(C.c_char_p), i64p, i64p, dp, i64p,
                                               C.POINTER(C.c_int32), i64p, C.c_int, dp]
            L.orc_adjoint_jacobian.restype = C.c_int
            L.orc_set_num_threads.argtypes = [C.c_int]
            L.orc_get_num_threads.restype = C.c_int
            _lib = L
    return _lib


def _check_state(sv):
    if not (isinstance(sv, np.ndarray) and sv.dtype == np.complex128 and sv.flags.c_contiguous):
        raise OracleError("oracle states are C-contiguous complex128 numpy arrays")
    n = int(sv.size).bit_length() - 1
    if sv.size != (1 << n):
        raise OracleError("state length must be a power of two")
    return n


def _i64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64).reshape(-1))


def _ptr(a, t=None):
    if t is None:
        return a.ctypes.data_as(C.c_void_p)
    return a.ctypes.data_as(C.POINTER(t))


def set_num_threads(n: int) -> None:
    lib().orc_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_get_num_threads())


def zero_state(nq: int) -> np.ndarray:
    sv = np.zeros(1 << nq, dtype=np.complex128)
    sv[0] = 1.0
    return sv


def apply(sv, name, wires, inverse=False, params=()):
    nq = _check_state(sv)
    w = _i64(wires)
    p = np.ascontiguousarray(np.asarray(params, dtype=np.float64).reshape(-1))
    st = lib().orc_apply(_ptr(sv), nq, name.encode(), _ptr(w, C.c_int64), len(w), int(bool(inverse)),
                         _ptr(p, C.c_double), len(p))
    if st != 0:
        raise OracleError(f"orc_apply({name}, {list(wires)}) -> {st}")
    return sv


def apply_matrix(sv, matrix, wires, inverse=False, refmap=False):
    nq = _check_state(sv)
    m = np.ascontiguousarray(np.asarray(matrix, dtype=np.complex128).reshape(-1))
    w = _i64(wires)
    if m.size != (1 << (2 * len(w))):
        raise OracleError("matrix size does not match the wire count")
    fn = lib().orc_apply_matrix_refmap if refmap else lib().orc_apply_matrix
    st = fn(_ptr(sv), nq, _ptr(m), _ptr(w, C.c_int64), len(w), int(bool(inverse)))
    if st != 0:
        raise OracleError(f"orc_apply_matrix -> {st}")
    return sv


def apply_generator(sv, name, wires, adj=False):
    nq = _check_state(sv)
    w = _i64(wires)
    st = C.c_int(0)
    s = lib().orc_apply_generator(_ptr(sv), nq, name.encode(), _ptr(w, C.c_int64), len(w), int(bool(adj)),
                                  C.byref(st))
    if st.value != 0:
        raise OracleError(f"orc_apply_generator({name}) -> {st.value}")
    return float(s)


def expval_named(sv, name, wires):
    nq = _check_state(sv)
    w = _i64(wires)
    st = C.c_int(0)
    r = lib().orc_expval_named(_ptr(sv), nq, name.encode(), _ptr(w, C.c_int64), len(w), C.byref(st))
    if st.value != 0:
        raise OracleError(f"orc_expval_named({name}) -> {st.value}")
    return float(r)


def expval_matrix(sv, matrix, wires):
    nq = _check_state(sv)
    m = np.ascontiguousarray(np.asarray(matrix, dtype=np.complex128).reshape(-1))
    w = _i64(wires)
    st = C.c_int(0)
    r = lib().orc_expval_matrix(_ptr(sv), nq, _ptr(m), _ptr(w, C.c_int64), len(w), C.byref(st))
    if st.value != 0:
        raise OracleError(f"orc_expval_matrix -> {st.value}")
    return float(r)


def expval_sparse(sv, data, indices, indptr):
    _check_state(sv)
    d = np.ascontiguousarray(np.asarray(data, dtype=np.complex128))
    ind, ptr = _i64(indices), _i64(indptr)
    return float(lib().orc_expval_sparse(_ptr(sv), len(ptr) - 1, _ptr(d), _ptr(ind, C.c_int64),
                                         _ptr(ptr, C.c_int64)))


def axpy(alpha, x, y):
    a = _Cplx(complex(alpha).real, complex(alpha).imag)
    lib().orc_axpy(a, _ptr(x), _ptr(y), x.size)
    return y


def spmv(x, data, indices, indptr):
    d = np.ascontiguousarray(np.asarray(data, dtype=np.complex128))
    ind, ptr = _i64(indices), _i64(indptr)
    y = np.zeros(len(ptr) - 1, dtype=np.complex128)
    lib().orc_spmv(_ptr(x), _ptr(y), len(ptr) - 1, _ptr(d), _ptr(ind, C.c_int64), _ptr(ptr, C.c_int64))
    return y


def inner_re(x, y):
    return float(lib().orc_inner_re(_ptr(x), _ptr(y), x.size))


def inner_im(x, y):
    return float(lib().orc_inner_im(_ptr(x), _ptr(y), x.size))


def probs(sv, wires=None):
    nq = _check_state(sv)
    if wires is None or len(wires) == 0 or (len(wires) == nq and list(wires) == sorted(wires)):
        out = np.empty(sv.size, dtype=np.float64)
        lib().orc_probs(_ptr(sv), nq, _ptr(out, C.c_double))
        return out
    w = _i64(wires)
    out = np.empty(1 << len(w), dtype=np.float64)
    st = lib().orc_probs_wires(_ptr(sv), nq, _ptr(w, C.c_int64), len(w), _ptr(out, C.c_double))
    if st != 0:
        raise OracleError("orc_probs_wires failed")
    return out


def cdf_exclusive(p):
    p = np.ascontiguousarray(p, dtype=np.float64)
    out = np.empty_like(p)
    lib().orc_cdf_exclusive(_ptr(p, C.c_double), p.size, _ptr(out, C.c_double))
    return out


def sample_from_uniforms(cdf, nq, uniforms):
    cdf = np.ascontiguousarray(cdf, dtype=np.float64)
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    out = np.empty((u.size, nq), dtype=np.int64)
    lib().orc_sample_from_uniforms(_ptr(cdf, C.c_double), cdf.size, nq, _ptr(u, C.c_double), u.size,
                                   _ptr(out, C.c_int64))
    return out


# --------------------------------------------------------------------------
# observables and the adjoint Jacobian
# --------------------------------------------------------------------------
def apply_observable(sv, obs):
    """O|sv> in place, following ObservablesKokkos.hpp applyInPlace."""
    kind = obs[0]
    if kind == "named":
        _, name, wires = obs
        if name != "Identity":
            apply(sv, name, wires, False, ())
    elif kind == "hermitian":
        _, matrix, wires = obs
        apply_matrix(sv, matrix, wires, False)
    elif kind == "tensor":
        for o in obs[1]:
            apply_observable(sv, o)
    elif kind == "hamiltonian":
        _, coeffs, terms = obs
        buf = np.zeros_like(sv)
        for c, t in zip(coeffs, terms):
            tmp = sv.copy()
            apply_observable(tmp, t)
            axpy(complex(c, 0.0), tmp, buf)
        sv[:] = buf
    elif kind == "sparse":
        _, data, indices, indptr, _wires = obs
        sv[:] = spmv(sv, data, indices, indptr)
    else:
        raise OracleError(f"unknown observable kind {kind}")
    return sv


def expval_observable(sv, obs):
    """MeasuresKokkos::expval(ob): Re<sv|O sv> (MeasuresKokkos.hpp:354-360)."""
    tmp = sv.copy()
    apply_observable(tmp, obs)
    return inner_re(sv, tmp)


def var_observable(sv, obs):
    """MeasuresKokkos::var(ob) (MeasuresKokkos.hpp:368-381)."""
    tmp = sv.copy()
    apply_observable(tmp, obs)
    return inner_re(tmp, tmp) - inner_re(sv, tmp) ** 2


def run_ops(sv, ops, adjoint=False):
    """Apply an op list [(name, wires, inverse, params)] (applyOperations)."""
    seq = reversed(ops) if adjoint else ops
    for name, wires, inv, params in seq:
        apply(sv, name, wires, bool(inv) ^ adjoint, params)
    return sv


def adjoint_jacobian(state, observables, ops, trainable):
    """AdjointJacobianKokkos::adjointJacobian (AdjointDiffKokkos.hpp:404-478)
    with apply_operations = false: `state` is the forward-evolved state.
    Returns jac[num_obs][num_trainable]."""
    nq = _check_state(state)
    hl = []
    for o in observables:
        h = state.copy()
        apply_observable(h, o)
        hl.append(h)
    names = [op[0].encode() for op in ops]
    wires, woff, params, poff, invs = [], [0], [], [0], []
    for name, w, inv, p in ops:
        wires.extend(int(x) for x in w)
        woff.append(len(wires))
        params.extend(float(x) for x in p)
        poff.append(len(params))
        invs.append(int(bool(inv)))
    w_a, woff_a, poff_a = _i64(wires if wires else [0]), _i64(woff), _i64(poff)
    p_a = np.ascontiguousarray(np.asarray(params if params else [0.0], dtype=np.float64))
    inv_a = np.ascontiguousarray(np.asarray(invs if invs else [0], dtype=np.int32))
    tp = _i64(trainable if len(trainable) else [0])
    jac = np.zeros((len(observables), len(trainable)), dtype=np.float64)
    name_arr = (C.c_char_p * max(1, len(names)))(*names)
    hl_arr = (C.c_void_p * max(1, len(hl)))(*[h.ctypes.data for h in hl])
    st = lib().orc_adjoint_jacobian(_ptr(state), nq, hl_arr, len(hl), len(ops), name_arr,
                                    _ptr(w_a, C.c_int64), _ptr(woff_a, C.c_int64), _ptr(p_a, C.c_double),
                                    _ptr(poff_a, C.c_int64), _ptr(inv_a, C.c_int32), _ptr(tp, C.c_int64),
                                    len(trainable), _ptr(jac, C.c_double))
    if st != 0:
        raise OracleError(f"orc_adjoint_jacobian -> {st}")
    return jac
