"""The allocation-free expectation-value entry point (plk_expval_pauliz_noalloc).

It serves callers that may not allocate device memory (their memory belongs to
another allocator or a fixed budget): it reads a caller-owned device state and
writes into a caller-owned device buffer, using a fixed library scratch array.
Checked through the C ABI against the allocating entry point
(plk_expval_named_batch) on two calls in a row, within the expectation-value
tolerances of the other tests (1e-10 complex128, 1e-5 complex64).  This file
is collected last so that a failure here does not stop the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

from abi import State, i64
from pennylane_lightning_kokkos import _native as N

pytestmark = pytest.mark.gpu

ETOL = {N.PLK_C128: 1e-10, N.PLK_C64: 1e-5}


def rand_state(nq, rng):
    v = rng.normal(size=1 << nq) + 1j * rng.normal(size=1 << nq)
    return v / np.linalg.norm(v)


def allocating_reference(state, wires):
    gates = np.array([N.GATE_ID["Identity"] if w < 0 else N.GATE_ID["PauliZ"] for w in wires], dtype=np.int32)
    w, wp = i64([max(x, 0) for x in wires])
    out = np.zeros(len(wires))
    N.check(N.lib.plk_expval_named_batch(state.h, len(wires), gates.ctypes.data_as(C.POINTER(C.c_int32)), wp,
                                         out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


def device_ptr(state):
    p = C.c_void_p()
    N.check(N.lib.plk_state_get(state.h, None, None, C.byref(p)))
    return p


# value counts: the maximum (16) and counts that fill only part of the kernel
# variant they run on (1, 3 -> 4, 5 -> 8, 9 -> 16), and the Identity alone
WIRE_SETS = {
    "16": list(range(15)) + [-1],
    "1": [7],
    "3": [0, 14, 6],
    "5": [3, -1, 12, 1, 9],
    "9": [8, 0, 2, 13, -1, 5, 11, 4, 14],
    "identity": [-1],
}


@pytest.mark.parametrize("dtype", [N.PLK_C128, N.PLK_C64])
@pytest.mark.parametrize("case", sorted(WIRE_SETS))
def test_noalloc_matches_allocating_entry_point(dtype, case):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(42)
    nq = 15
    wires = WIRE_SETS[case]
    out = torch.full((len(wires),), float("nan"), dtype=torch.float64, device="cuda")
    w, wp = i64(wires)
    for call in range(2):  # two calls in a row share the scratch array
        st = State.from_array(rand_state(nq, rng), dtype)
        ref = allocating_reference(st, wires)
        N.check(N.lib.plk_state_synchronize(st.h))
        N.check(N.lib.plk_expval_pauliz_noalloc(device_ptr(st), nq, dtype, len(wires), wp,
                                                C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_double)),
                                                C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got, ref, atol=ETOL[dtype], rtol=0, err_msg=f"call {call}")
        for i, wi in enumerate(wires):
            if wi < 0:  # Identity: the squared norm of a normalised state
                assert abs(got[i] - 1.0) < ETOL[dtype]


def test_noalloc_rejects_too_many_values():
    torch = pytest.importorskip("torch")
    st = State(4)
    out = torch.zeros(17, dtype=torch.float64, device="cuda")
    w, wp = i64([0] * 17)
    status = N.lib.plk_expval_pauliz_noalloc(device_ptr(st), 4, N.PLK_C128, 17, wp,
                                             C.cast(C.c_void_p(out.data_ptr()), C.POINTER(C.c_double)), None)
    assert status == 1 and "at most 16 values" in N.last_error()
