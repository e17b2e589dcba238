#!/usr/bin/env python3
"""Gate-throughput benchmark of the GB300 state-vector core.

Workload (one GPU): the gate-throughput sweep on a 30-qubit complex128 state
(16 GiB, wire 0 = most significant bit) prepared by a Hadamard layer.  One
step applies, for each of PauliX, Hadamard, RX, CNOT, CRY, IsingXX,
SingleExcitation, DoubleExcitation and a Haar-random two-qubit matrix, `reps`
applications on distinct wires drawn from each of the low (0-4), mid (12-17)
and high (25-29) wire ranges, angles uniform in [0, 2*pi) (seed 2).

Metric: algorithmic HBM GB/s = sum over applications of touched_fraction x
2 x 2^30 x 16 B (read + write) / device time.  The state (16 GiB) is far
larger than L2 (129 MB), so no L2 flush is needed between applications.

Printed JSON line:
  value      - device-resident throughput (CUDA events on the state's stream)
  e2e        - the same metric through the reference-facing pybind API
               (LightningKokkos_C128) with the state copied from pinned host
               memory before and back after every step: three states on
               three streams take steps in turn, so a step's copies overlap
               other steps' gates (`serial`: one state, blocking copies)
  roofline   - the gate kernel with the largest time share, against the
               measured HBM copy bandwidth
  per_gate   - GB/s and time share of every gate type (and wire range)
  per_gate_fp64 - the same step with complex128 kernels in native IEEE FP64
               arithmetic (the default is double-float on the FP32 pipe;
               `dtype` says which ran)
  cpu_baseline - the oracle (CPU restatement of the reference functors) on
               the host cores, one application per gate type and wire range
  parity     - the GPU path against the oracle at the benchmarked sizes: the
               30-qubit state after the cpu_baseline applications, the
               26-qubit adjoint gradients (2 layers; all 40 with --only parity,
               which also runs 31- and 32-qubit circuits), the 20-qubit
               Jacobian
  adjoint_26q - adjoint Jacobian of the 26-qubit ansatz (40 layers of RY, RZ
               + CNOT ladder, 100-term Pauli Hamiltonian) in complex64 with
               FP64 accumulation vs complex128, seconds per gradient and the
               largest gradient difference
  batch      - 4096 circuits (8-20 qubits, 5-30 layers, 10-term Hamiltonians),
               forward + <H> + adjoint gradient in one persistent complex64
               launch replayed as a CUDA graph (autotuned), circuits/s,
               against a per-circuit loop of the plain path and the oracle
  plain_20q  - 20-qubit complex128 circuit (600 parameters), 20 <PauliZ> and
               the 20 x 600 Jacobian through the reference-facing module,
               against the oracle on the host cores
  precision  - 32-qubit complex64 vs 31-qubit complex128 at equal bytes,
               200-word Hamiltonian, error against complex128
`--impl reference` times the oracle (the CPU restatement of the reference
functors) on the host cores instead.  For --gpus N
under torchrun every rank runs an independent replica (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes as C
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "pennylane-lightning-kokkos_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

METRIC = "gate HBM GB/s vs peak; adjoint grad s/circuit c64+FP64-acc vs c128 at stated err"
# what bounds a gate kernel below the HBM roofline (from its ncu profile)
KERNEL_LIMITS = {
    "Haar2q": "FP32-pipe issue: the complex128 4x4 matrix runs in double-float, 16 error-free multiply-adds "
              "per amplitude with the real and imaginary lanes packed two per instruction (.f32x2); DRAM "
              "traffic equals the algorithmic bytes; the complex64 kernel runs at the copy rate",
}
GIB = 1 << 30


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--nq", type=int, default=30)
    ap.add_argument("--reps", type=int, default=4,
                    help="applications per gate and wire range per step (the reference arm times one per step)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--adjoint-nq", type=int, default=26)
    ap.add_argument("--adjoint-layers", type=int, default=40)
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-circuits", type=int, default=4096)
    ap.add_argument("--no-plain20", action="store_true")
    ap.add_argument("--only", choices=["adjoint", "batch", "plain20", "precision", "kernels", "parity"],
                    default=None, help="run one secondary config alone and print its JSON (profiling, spot checks, "
                                       "and the full-size oracle parity run)")
    ap.add_argument("--no-tune", action="store_true", help="batch: fixed launch configuration instead of autotuning")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the equal-bytes precision config (32-qubit complex64 vs 31-qubit complex128)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the native-FP64 pass of the gate sweep")
    ap.add_argument("--parity-layers", type=int, default=None,
                    help="layers of the 26-qubit adjoint parity check against the oracle (default: 2 in the main "
                         "run, 40 with --only parity)")
    ap.add_argument("--census-nq", type=int, default=26, help="--only kernels: state size in qubits")
    ap.add_argument("--census-reps", type=int, default=3, help="--only kernels: timed calls per entry point")
    return ap.parse_args(argv)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------- clocks --
class ClockSampler:
    FIELDS = ["index", "clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device):
        self.device, self.lines, self.proc, self.err = device, [], None, None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + ",".join(self.FIELDS), "--format=csv,noheader,nounits", "-lms",
                 "200", "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception as e:  # nvidia-smi missing
            self.err = str(e)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"unavailable": self.err or "nvidia-smi not started"}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"unavailable": "no samples"}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ device sweep --
class SweepRunner:
    """Applies a gate-sweep plan to a device-resident state through the C ABI."""

    def __init__(self, nq, plan, device, stream):
        from pennylane_lightning_kokkos import _native as N

        self.N, self.nq, self.plan = N, nq, plan
        h = C.c_void_p()
        N.check(N.lib.plk_state_create(nq, N.PLK_C128, device, C.byref(h)))
        self.h = h
        N.check(N.lib.plk_state_set_stream(h, C.c_void_p(stream.cuda_stream)))
        self.keep, self.calls = [], []
        for app in plan:
            w = np.array(app["wires"], dtype=np.int64)
            self.keep.append(w)
            wp = w.ctypes.data_as(C.POINTER(C.c_int64))
            if app["matrix"] is not None:
                m = np.ascontiguousarray(app["matrix"], dtype=np.complex128)
                self.keep.append(m)
                self.calls.append(("m", m.ctypes.data_as(C.POINTER(C.c_double)), wp, len(w)))
            else:
                p = np.array(app["params"] or [0.0], dtype=np.float64)
                self.keep.append(p)
                self.calls.append(("g", N.GATE_ID[app["name"]], wp, len(w), p.ctypes.data_as(C.POINTER(C.c_double)),
                                   len(app["params"])))
        # |+>^n: Hadamard on every wire
        for wire in range(nq):
            w = np.array([wire], dtype=np.int64)
            N.check(N.lib.plk_apply_gate(h, N.GATE_ID["Hadamard"], w.ctypes.data_as(C.POINTER(C.c_int64)), 1, 0,
                                         None, 0))

    def apply(self, i):
        c = self.calls[i]
        if c[0] == "m":
            st = self.N.lib.plk_apply_matrix(self.h, c[1], c[2], c[3], 0)
        else:
            st = self.N.lib.plk_apply_gate(self.h, c[1], c[2], c[3], 0, c[4], c[5])
        if st:
            self.N.check(st)

    def close(self):
        self.N.lib.plk_state_destroy(self.h)


def run_device_sweep(args, device, torch, dist_barrier):
    from pennylane_lightning_kokkos.circuits import gate_sweep_plan

    plan = gate_sweep_plan(args.nq, args.reps, seed=2)
    stream = torch.cuda.Stream(device=device)
    runner = SweepRunner(args.nq, plan, device, stream)
    amp = 2 * (1 << args.nq) * 16  # bytes read + written for the full state
    groups = []  # (gate name, [plan indices])
    for i, app in enumerate(plan):
        if not groups or groups[-1][0] != app["name"]:
            groups.append((app["name"], []))
        groups[-1][1].append(i)
    range_groups = {}
    for i, app in enumerate(plan):
        range_groups.setdefault((app["name"], app["range"]), []).append(i)

    def step(events=None):
        for gi, (_, idx) in enumerate(groups):
            if events is not None:
                events[gi].record(stream)
            for i in idx:
                runner.apply(i)
        if events is not None:
            events[-1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(device)
    clocks = ClockSampler(device)
    clocks.start()
    time.sleep(0.3)
    dist_barrier()
    torch.cuda.synchronize(device)
    mk = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    t0, t1 = mk(), mk()
    step_events = [[mk() for _ in range(len(groups) + 1)] for _ in range(args.steps)]
    t0.record(stream)
    for k in range(args.steps):
        step(step_events[k])
    t1.record(stream)
    torch.cuda.synchronize(device)
    dist_barrier()
    clk = clocks.stop()
    total_ms = t0.elapsed_time(t1)
    per_gate_ms = {g: 0.0 for g, _ in groups}
    for k in range(args.steps):
        ev = step_events[k]
        for gi, (g, _) in enumerate(groups):
            per_gate_ms[g] += ev[gi].elapsed_time(ev[gi + 1])
    bytes_per_gate = {g: sum(plan[i]["touched"] * amp for i in idx) * args.steps for g, idx in groups}
    total_bytes = sum(bytes_per_gate.values())
    # per (gate, range) timing: one extra untimed-for-value pass with events per range
    rng_ms = {}
    ev = {key: (mk(), mk()) for key in range_groups}
    for key, idx in range_groups.items():
        ev[key][0].record(stream)
        for i in idx:
            runner.apply(i)
        ev[key][1].record(stream)
    torch.cuda.synchronize(device)
    for key, (a, b) in ev.items():
        ms = a.elapsed_time(b)
        nbytes = sum(plan[i]["touched"] * amp for i in range_groups[key])
        rng_ms[f"{key[0]}/{key[1]}"] = {"ms_per_app": ms / len(range_groups[key]),
                                       "GBps": nbytes / (ms * 1e6)}
    fp64 = None if args.no_fp64 else fp64_pass(runner, groups, plan, amp, stream, torch, device)
    runner.close()
    return {
        "plan": plan, "groups": groups, "total_ms": total_ms, "per_gate_ms": per_gate_ms,
        "bytes_per_gate": bytes_per_gate, "total_bytes": total_bytes, "clocks": clk, "per_range": rng_ms,
        "launches": len(plan) * args.steps, "fp64": fp64,
    }


def fp64_pass(runner, groups, plan, amp, stream, torch, device):
    """The same step with the complex128 kernels in native IEEE FP64
    arithmetic instead of double-float (one warm-up step, one timed step):
    the comparison figure for the double-float default."""
    N = runner.N
    before = N.c128_arithmetic()
    N.set_c128_arithmetic("fp64")
    mk = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    try:
        for _, idx in groups:
            for i in idx:
                runner.apply(i)
        torch.cuda.synchronize(device)
        ev = [mk() for _ in range(len(groups) + 1)]
        for gi, (_, idx) in enumerate(groups):
            ev[gi].record(stream)
            for i in idx:
                runner.apply(i)
        ev[-1].record(stream)
        torch.cuda.synchronize(device)
    finally:
        N.set_c128_arithmetic(before)
    per_gate, tot_ms, tot_b = {}, 0.0, 0.0
    for gi, (g, idx) in enumerate(groups):
        ms = ev[gi].elapsed_time(ev[gi + 1])
        nbytes = sum(plan[i]["touched"] * amp for i in idx)
        per_gate[g] = {"GBps": nbytes / (ms * 1e6), "ms_per_app": ms / len(idx)}
        tot_ms += ms
        tot_b += nbytes
    return {"value": tot_b / (tot_ms * 1e6), "unit": "GB/s", "per_gate": per_gate,
            "arithmetic": "native IEEE FP64 (complex128), one timed step"}


# -------------------------------------------------------------------- e2e --
def run_e2e(args, device, torch, plan, steps):
    """The sweep through the reference-facing module with host buffers: every
    step copies a 2^n complex128 state in from pinned host memory, applies the
    step's gates and copies the result back out.

    Pipelined (the reported value): three states, each on its own CUDA
    stream, take steps in turn; copies are queued (HostToDeviceAsync /
    DeviceToHostAsync) and each step's gates start after the previous step's,
    so a state's copies out and in run while the other two states' gates do
    (two gate periods of slack for a host link whose rate varies).  Serial: one state, the blocking HostToDevice / DeviceToHost of the
    reference API, one step at a time."""
    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m

    n = 1 << args.nq
    amp = 2 * n * 16
    step_bytes = sum(a["touched"] * amp for a in plan)
    names = [a["name"] for a in plan]
    inp = torch.empty(n, dtype=torch.complex128, pin_memory=True).numpy()
    inp[:] = 1.0 / np.sqrt(n)
    P = 3  # states in the pipeline
    outs = [torch.empty(n, dtype=torch.complex128, pin_memory=True).numpy() for _ in range(P)]

    def gates(sv):
        for a in plan:
            if a["matrix"] is not None:
                sv.apply("QubitUnitary", a["wires"], False, [[]], a["matrix"])
            else:
                getattr(sv, a["name"])(a["wires"], False, a["params"])

    settings = m.InitializationSettings().set_device_id(device)
    # serial: the reference API's blocking copies
    sv = m.LightningKokkos_C128(args.nq, settings)

    def serial_step():
        sv.HostToDevice(inp)
        gates(sv)
        sv.DeviceToHost(outs[0])

    serial_step()  # warm-up
    t = time.perf_counter()
    for _ in range(steps):
        serial_step()
    serial_s = (time.perf_counter() - t) / steps
    del sv
    # pipelined: P states on P streams
    streams = [torch.cuda.Stream(device=device) for _ in range(P)]
    svs = [m.LightningKokkos_C128(args.nq, settings) for _ in range(P)]
    for k in range(P):
        svs[k].set_stream(streams[k].cuda_stream)

    # a step's gates wait for the previous step's gates (an event between the
    # streams): the states never compete for the SMs, so a state's copies run
    # while the others' gates do instead of all copying at once
    done = [torch.cuda.Event() for _ in range(P)]

    def queue_step(k):
        i = k % P
        s = svs[i]
        s.HostToDeviceAsync(inp)
        if k > 0:
            streams[i].wait_event(done[(k - 1) % P])
        gates(s)
        done[i].record(streams[i])
        s.DeviceToHostAsync(outs[i])

    for k in range(P):  # warm-up
        queue_step(k)
    for s in svs:
        s.synchronize()
    psteps = max(10, 2 * steps)  # the first copy in and the last copy out are not overlapped: amortise them
    t = time.perf_counter()
    for k in range(psteps):
        queue_step(k)
    for s in svs:
        s.synchronize()
    pipe_s = (time.perf_counter() - t) / psteps
    del svs
    del inp, outs  # release the pinned buffers (torch caches them otherwise)
    gc.collect()
    if hasattr(torch._C, "_host_emptyCache"):
        torch._C._host_emptyCache()
    return {"value": step_bytes / pipe_s / 1e9, "unit": "GB/s", "h2d_bytes_per_step": n * 16,
            "d2h_bytes_per_step": n * 16, "steps": psteps, "s_per_step": pipe_s,
            "api": "lightning_kokkos_qubit_ops.LightningKokkos_C128: HostToDeviceAsync, gates, DeviceToHostAsync "
                   "(pinned host buffers)",
            "pipeline": f"{P} states on {P} CUDA streams take steps in turn; each step's gates wait for the previous "
                        "step's, and a state's copies overlap the other states' gates; host wall clock from the first "
                        "queued copy to the last result in host memory",
            "serial": {"value": step_bytes / serial_s / 1e9, "s_per_step": serial_s, "steps": steps,
                       "api": "LightningKokkos_C128.HostToDevice, gates, DeviceToHost (blocking, one state)"},
            "gates_per_step": len(names)}


# ------------------------------------------------------------- CPU legs --
def oracle_apply_plan(sv, plan):
    import oracle as O

    for a in plan:
        if a["matrix"] is not None:
            O.apply_matrix(sv, a["matrix"], a["wires"])
        else:
            O.apply(sv, a["name"], a["wires"], False, a["params"])
    return sv


def oracle_sweep(nq, plan, threads):
    """The oracle on |+>^n through `plan`: (GB/s, seconds, final state)."""
    import oracle as O

    O.set_num_threads(threads)
    n = 1 << nq
    sv = np.full(n, 1.0 / np.sqrt(n), dtype=np.complex128)
    t = time.perf_counter()
    oracle_apply_plan(sv, plan)
    dt = time.perf_counter() - t
    nbytes = sum(a["touched"] * 2 * n * 16 for a in plan)
    return nbytes / dt / 1e9, dt, sv


def run_cpu_baseline(args):
    """The oracle on the host cores, one application per gate type and wire
    range (27); also returns its final state and plan for the parity check."""
    from pennylane_lightning_kokkos.circuits import gate_sweep_plan

    threads = os.cpu_count() or 1
    plan = gate_sweep_plan(args.nq, 1, seed=2)
    gbs, dt, sv = oracle_sweep(args.nq, plan, threads)
    return {"value": gbs, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"{len(plan)} applications (1 per gate x wire range) on the {args.nq}-qubit complex128 "
                      f"state, OpenMP oracle, {dt:.1f} s"}, sv, plan


def max_abs_diff_chunked(a, b, chunk=1 << 26):
    """max |a - b| over two large host arrays, a chunk at a time"""
    m = 0.0
    for off in range(0, a.size, chunk):
        x = a[off:off + chunk].astype(np.complex128, copy=False)
        m = max(m, float(np.max(np.abs(x - b[off:off + chunk]))))
    return m


def gpu_state_after(nq, dtype, device, prepare, plan=None, ops=None):
    """Device state: `prepare` (a list of gate ops through plk_apply_ops, or
    'hadamard' for H on every wire), then `plan` (sweep applications, one
    C-ABI call each) or `ops` (one plk_apply_ops call); returned on the host."""
    from pennylane_lightning_kokkos import _native as N

    h = C.c_void_p()
    N.check(N.lib.plk_state_create(nq, dtype, device, C.byref(h)))
    keep = []

    def apply_ops(lst):
        arr = (N.PlkOp * len(lst))()
        for i, (name, w, inv, p) in enumerate(lst):
            wa = np.array(w, dtype=np.int64)
            pa = np.array(p or [0.0], dtype=np.float64)
            keep.extend([wa, pa])
            arr[i] = N.PlkOp(N.GATE_ID[name], len(w), int(inv), len(p), wa.ctypes.data_as(C.POINTER(C.c_int64)),
                             pa.ctypes.data_as(C.POINTER(C.c_double)), None)
        N.check(N.lib.plk_apply_ops(h, arr, len(lst)))

    try:
        if prepare == "hadamard":
            w = np.zeros(1, dtype=np.int64)
            for wire in range(nq):
                w[0] = wire
                N.check(N.lib.plk_apply_gate(h, N.GATE_ID["Hadamard"], w.ctypes.data_as(C.POINTER(C.c_int64)), 1, 0,
                                             None, 0))
        elif prepare:
            apply_ops(prepare)
        for a in plan or []:
            wa = np.array(a["wires"], dtype=np.int64)
            wp = wa.ctypes.data_as(C.POINTER(C.c_int64))
            if a["matrix"] is not None:
                m = np.ascontiguousarray(a["matrix"], dtype=np.complex128)
                N.check(N.lib.plk_apply_matrix(h, m.ctypes.data_as(C.POINTER(C.c_double)), wp, len(wa), 0))
            else:
                p = np.array(a["params"] or [0.0], dtype=np.float64)
                N.check(N.lib.plk_apply_gate(h, N.GATE_ID[a["name"]], wp, len(wa), 0,
                                             p.ctypes.data_as(C.POINTER(C.c_double)), len(a["params"])))
        if ops:
            apply_ops(ops)
        out = np.empty(1 << nq, dtype=np.complex128 if dtype == N.PLK_C128 else np.complex64)
        N.check(N.lib.plk_state_d2h(h, out.ctypes.data_as(C.c_void_p), out.size))
    finally:
        N.lib.plk_state_destroy(h)
    return out


def sweep_parity(args, device, sv_ref, plan):
    """The GPU path on the same applications as the oracle leg, from |+>^n:
    max |psi_gpu - psi_oracle| over all 2^n amplitudes (bar: 1e-12)."""
    from pennylane_lightning_kokkos import _native as N

    t = time.perf_counter()
    got = gpu_state_after(args.nq, N.PLK_C128, device, "hadamard", plan=plan)
    d = max_abs_diff_chunked(got, sv_ref)
    del got
    return {"qubits": args.nq, "applications": len(plan), "max_abs_state_diff_vs_oracle": d, "tolerance": 1e-12,
            "pass": d <= 1e-12, "arithmetic": N.c128_arithmetic(), "seconds": time.perf_counter() - t}


def sweep_config(args):
    """The `config` of both arms: the workload whose rate both measure (a step
    of either arm applies every gate type on every wire range equally often;
    the arms differ only in how many applications a step holds, `step_plan`)."""
    return {"workload": f"gate sweep, {args.nq} qubits complex128 ({(1 << args.nq) * 16 / GIB:.0f} GiB state), "
                        "9 gate types x low/mid/high wire ranges, equal counts, seed 2",
            "l2": "state larger than L2 (129 MB): no flush needed"}


def run_reference_arm(args, rank):
    """--impl reference: the oracle (plain-C restatement of the reference's
    Kokkos functors, OpenMP on every host core) on the sweep workload, one
    application per gate type and wire range per step, from |+>^n."""
    from pennylane_lightning_kokkos.circuits import gate_sweep_plan

    if rank != 0:
        return None
    import oracle as O

    threads = os.cpu_count() or 1
    O.set_num_threads(threads)
    plan = gate_sweep_plan(args.nq, 1, seed=2)  # one application per gate type and wire range
    n = 1 << args.nq
    sv = np.full(n, 1.0 / np.sqrt(n), dtype=np.complex128)
    for _ in range(args.warmup):
        oracle_apply_plan(sv, plan)
    t = time.perf_counter()
    for _ in range(args.steps):
        oracle_apply_plan(sv, plan)
    dt = time.perf_counter() - t
    nbytes = sum(a["touched"] * 2 * n * 16 for a in plan) * args.steps
    value = nbytes / dt / 1e9
    return {
        "metric": METRIC, "value": value, "unit": "GB/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / max(1, args.steps),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "complex128 (native FP64, CPU oracle)", "data": "synthetic (seeded gate sweep, seed 2)",
        "config": sweep_config(args),
        "step_plan": f"{len(plan)} applications: 1 per gate type and wire range, the same every step",
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} steps x {len(plan)} applications (one per gate type and wire "
                                   "range), OpenMP oracle"},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ------------------------------------------------------------ adjoint 26q --
def module_gradient_fn(m, bits, device, nq, ops, words):
    """A callable that runs one adjoint gradient of <H> through the
    reference-facing module (state, tape, Hamiltonian of Pauli words)."""
    dt = np.float64 if bits == "128" else np.float32
    cdt = np.complex128 if bits == "128" else np.complex64
    L = lambda name: getattr(m, name + "_C" + bits)  # noqa: E731
    ham = _words_obs(m, bits, words)
    adj = L("AdjointJacobianKokkos")()
    tape = adj.create_ops_list([o[0] for o in ops], [np.array(o[3], dtype=dt) for o in ops], [o[1] for o in ops],
                               [o[2] for o in ops], [np.array([], dtype=cdt)] * len(ops))
    names, wires, invs, prms = [o[0] for o in ops], [o[1] for o in ops], [o[2] for o in ops], [o[3] for o in ops]
    npar = sum(1 for o in ops if o[3])

    def gradient():
        sv = L("LightningKokkos")(nq, m.InitializationSettings().set_device_id(device))
        sv.apply(names, wires, invs, prms)
        return np.asarray(adj.adjoint_jacobian(sv, [ham], tape, list(range(npar))), dtype=np.float64)[0]

    return gradient


def run_adjoint(args, device, torch):
    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m
    from pennylane_lightning_kokkos.circuits import hardware_efficient_ansatz, random_pauli_words

    nq, layers = args.adjoint_nq, args.adjoint_layers
    ops = hardware_efficient_ansatz(nq, layers, seed=4, rotations=("RY", "RZ"), entangler="ladder")
    words = random_pauli_words(nq, 100, seed=4)
    npar = sum(1 for o in ops if o[3])
    out = {"qubits": nq, "layers": layers, "params": npar, "ops": len(ops), "hamiltonian_terms": len(words)}
    grads = {}
    for bits in ("128", "64"):
        gradient = module_gradient_fn(m, bits, device, nq, ops, words)
        gradient()  # warm-up (allocator pools, module load)
        torch.cuda.synchronize(device)
        reps = 2
        t = time.perf_counter()
        for _ in range(reps):
            g = gradient()
        torch.cuda.synchronize(device)
        out[f"c{bits}_s_per_gradient"] = (time.perf_counter() - t) / reps
        grads[bits] = g
    out["c64_speedup_vs_c128"] = out["c128_s_per_gradient"] / out["c64_s_per_gradient"]
    out["max_abs_grad_diff_c64_vs_c128"] = float(np.max(np.abs(grads["64"] - grads["128"])))
    out["error_reference"] = ("complex128 GPU path; both precisions against the FP64 oracle: the parity key "
                              "(2 layers here, all 40 layers with --only parity)")
    return out


def run_adjoint_parity(args, device, torch, layers):
    """The 26-qubit ansatz (RY, RZ on every wire + CNOT ladder, seed 4) with
    `layers` layers and the 100-term Hamiltonian: adjoint gradients through
    the module in complex128 and complex64 against the oracle's adjoint
    Jacobian (FP64, host cores).  Bars: complex128 1e-10, complex64 1e-5."""
    import oracle as O
    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m
    from pennylane_lightning_kokkos.circuits import hardware_efficient_ansatz, random_pauli_words

    nq = args.adjoint_nq
    ops = hardware_efficient_ansatz(nq, layers, seed=4, rotations=("RY", "RZ"), entangler="ladder")
    words = random_pauli_words(nq, 100, seed=4)
    npar = sum(1 for o in ops if o[3])
    grads = {bits: module_gradient_fn(m, bits, device, nq, ops, words)() for bits in ("128", "64")}
    torch.cuda.synchronize(device)
    threads = os.cpu_count() or 1
    O.set_num_threads(threads)
    letters = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}
    obs = ("hamiltonian", [c for c, _, _ in words],
           [("tensor", [("named", letters[x], [wi]) for wi, x in zip(w, l)]) for _, w, l in words])
    t = time.perf_counter()
    psi = O.run_ops(O.zero_state(nq), ops)
    ref = O.adjoint_jacobian(psi, [obs], ops, list(range(npar)))[0]
    del psi
    cpu_s = time.perf_counter() - t
    d128 = float(np.max(np.abs(grads["128"] - ref)))
    d64 = float(np.max(np.abs(grads["64"] - ref)))
    return {"qubits": nq, "layers": layers, "params": npar, "ops": len(ops), "hamiltonian_terms": len(words),
            "c128_max_abs_grad_diff_vs_oracle": d128, "c64_max_abs_grad_diff_vs_oracle": d64,
            "max_abs_grad_oracle": float(np.max(np.abs(ref))), "tolerance": {"c128": 1e-10, "c64": 1e-5},
            "pass": d128 <= 1e-10 and d64 <= 1e-5, "oracle_seconds": cpu_s, "oracle_cores": threads}


def run_large_index_parity(device, nq, dtype_name):
    """A short circuit at 31 qubits complex128 or 32 qubits complex64 (amplitude
    indices beyond 2^31; the register-window path at its 32-qubit limit):
    RY with seeded angles on every wire, then 12 ops on the highest, lowest
    and middle wires, through plk_apply_ops; the whole state against the
    oracle (FP64).  Bars: complex128 1e-12, complex64 5e-6."""
    import oracle as O
    from pennylane_lightning_kokkos import _native as N

    rng = np.random.default_rng(31)
    prep = [("RY", [w], False, [float(rng.uniform(0, np.pi))]) for w in range(nq)]
    a = lambda: [float(rng.uniform(0, 2 * np.pi))]  # noqa: E731
    lo, mid, hi = nq - 1, nq // 2, 0  # wire 0 is the most significant bit
    ops = [("RY", [hi], False, a()), ("CNOT", [hi, lo], False, []), ("RZ", [lo], False, a()),
           ("IsingXX", [hi, lo], False, a()), ("CRY", [lo, hi], False, a()), ("RX", [mid], False, a()),
           ("CNOT", [lo, 1], False, []), ("RZ", [hi], False, a()), ("SingleExcitation", [1, lo], False, a()),
           ("Hadamard", [hi], False, []), ("CZ", [hi, mid], False, []), ("RY", [lo], False, a())]
    dtype = N.PLK_C128 if dtype_name == "c128" else N.PLK_C64
    t = time.perf_counter()
    got = gpu_state_after(nq, dtype, device, prep, ops=ops)
    gpu_s = time.perf_counter() - t
    O.set_num_threads(os.cpu_count() or 1)
    t = time.perf_counter()
    ref = O.run_ops(O.zero_state(nq), prep + ops)
    cpu_s = time.perf_counter() - t
    d = max_abs_diff_chunked(got, ref)
    del got, ref
    tol = 1e-12 if dtype_name == "c128" else 5e-6
    return {"qubits": nq, "dtype": dtype_name, "ops": len(prep) + len(ops), "max_abs_state_diff_vs_oracle": d,
            "tolerance": tol, "pass": d <= tol, "gpu_seconds_with_d2h": gpu_s, "oracle_seconds": cpu_s}


def run_parity(args, device, torch):
    """--only parity: every oracle comparison at the benchmarked sizes (30-qubit
    sweep state, 26-qubit 40-layer adjoint gradients in both precisions,
    31-qubit complex128 and 32-qubit complex64 short circuits)."""
    layers = args.parity_layers or 40
    out = {}
    _, sv, plan = run_cpu_baseline(args)
    out["sweep_state"] = sweep_parity(args, device, sv, plan)
    del sv
    out["large_index_c128_31q"] = run_large_index_parity(device, 31, "c128")
    out["large_index_c64_32q"] = run_large_index_parity(device, 32, "c64")
    out["adjoint_26q"] = run_adjoint_parity(args, device, torch, layers)
    out["pass"] = all(v.get("pass", False) for v in out.values() if isinstance(v, dict))
    return out


# ---------------------------------------------------------- batching C5 --
def _words_obs(m, bits, words):
    letters = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}
    L = lambda name: getattr(m, name + "_C" + bits)  # noqa: E731
    dt = np.float64 if bits == "128" else np.float32
    terms = []
    for c, w, l in words:
        fac = [L("NamedObsKokkos")(letters[x], [wi]) for wi, x in zip(w, l)]
        terms.append(fac[0] if len(fac) == 1 else L("TensorProdObsKokkos")(fac))
    return L("HamiltonianKokkos")(np.array([c for c, _, _ in words], dtype=dt), terms)


def plain_circuit_gradient(m, bits, device, nq, ops, words):
    """One circuit through the reference-facing module: state, tape, <H>,
    adjoint Jacobian of every parameter (what the reference device does per tape)."""
    L = lambda name: getattr(m, name + "_C" + bits)  # noqa: E731
    dt = np.float64 if bits == "128" else np.float32
    cdt = np.complex128 if bits == "128" else np.complex64
    sv = L("LightningKokkos")(nq, m.InitializationSettings().set_device_id(device))
    names, wires, invs, prms = [o[0] for o in ops], [o[1] for o in ops], [o[2] for o in ops], [o[3] for o in ops]
    sv.apply(names, wires, invs, prms)
    ev = sv.ExpectationValuePauliSum([c for c, _, _ in words], [w for _, w, _ in words], [l for _, _, l in words])
    adj = L("AdjointJacobianKokkos")()
    tape = adj.create_ops_list(names, [np.array(p, dtype=dt) for p in prms], wires, invs,
                               [np.array([], dtype=cdt)] * len(ops))
    npar = sum(1 for p in prms if p)
    jac = np.asarray(adj.adjoint_jacobian(sv, [_words_obs(m, bits, words)], tape, list(range(npar))))[0]
    return ev, jac


def run_batch(args, device, torch):
    """Batching: forward + <H> + adjoint gradient of every circuit of a
    seeded uneven batch in one persistent complex64 launch (CUDA graph),
    against a per-circuit loop of the plain path and the oracle."""
    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m
    from pennylane_lightning_kokkos.batch import CircuitBatch
    from pennylane_lightning_kokkos.circuits import batch_workload_packed, packed_to_ops

    n = args.batch_circuits
    wl = batch_workload_packed(n, seed=5)
    work = np.array([len(pk["gates"]) * float(1 << nq) for nq, pk, _ in wl])
    gate_apps = sum(len(pk["gates"]) for _, pk, _ in wl)
    # autotune on a one-in-sixteen subsample, then run the whole batch with the winner
    if args.no_tune:
        report, tune_s = "not tuned", 0.0
        cfg = {"cluster": 8, "smem_qubits": 12, "cluster_min_qubits": 13, "ctas_per_sm": 2}
    else:
        sub = CircuitBatch("c64", device)
        for nq, pk, words in wl[::16]:
            sub.add_packed(nq, pk, words)
        t = time.perf_counter()
        report = sub.tune(reps=1)
        tune_s = time.perf_counter() - t
        cfg = sub.get_config()
        sub.close()
    b = CircuitBatch("c64", device)
    for nq, pk, words in wl:
        b.add_packed(nq, pk, words)
    b.set_config(cluster=cfg["cluster"], smem_qubits=cfg["smem_qubits"], cluster_min_qubits=cfg["cluster_min_qubits"],
                 ctas_per_sm=cfg["ctas_per_sm"])
    t = time.perf_counter()
    b.run()
    first_s = time.perf_counter() - t
    _, npar, njac = b.info()
    params = np.concatenate([pk["params"] for _, pk, _ in wl])
    b.run(params)
    dev_ms, wall_s = [], []
    for _ in range(3):
        t = time.perf_counter()
        ev, jac = b.run(params)
        wall_s.append(time.perf_counter() - t)
        dev_ms.append(b.last_time()[0])
    launches = b.last_time()[1]
    grads = b.gradients(jac)
    b.close()
    ms = statistics.median(dev_ms)
    out = {"circuits": n, "qubits": "uniform 8-20", "layers": "uniform 5-30 (RX, RY, RZ + CNOT ladder)",
           "hamiltonian_terms": 10, "dtype": "complex64 state, double-float accumulation",
           "params": int(npar), "gate_applications_forward": int(gate_apps),
           "tuned_config": cfg, "tune_seconds": tune_s, "first_run_seconds": first_s,
           "device_ms": ms, "circuits_per_s": n / (ms / 1e3),
           "e2e_circuits_per_s": n / statistics.median(wall_s),
           "e2e_api": "CircuitBatch.run (parameters in, <H> and gradients out, host arrays)",
           "gate_applications_per_s": gate_apps / (ms / 1e3), "kernel_launches_per_run": int(launches),
           "tune_report": report.strip().splitlines()}
    # accuracy: complex128 batch on a sample
    idx = list(range(0, n, max(1, n // 64)))
    b128 = CircuitBatch("c128", device)
    for i in idx:
        b128.add_packed(wl[i][0], wl[i][1], wl[i][2])
    ev128, jac128 = b128.run()
    g128 = b128.gradients(jac128)
    b128.close()
    out["max_abs_expval_diff_c64_vs_c128"] = float(max(abs(ev[i] - ev128[k]) for k, i in enumerate(idx)))
    out["max_abs_grad_diff_c64_vs_c128"] = float(max(np.max(np.abs(grads[i] - g128[k])) for k, i in enumerate(idx)))
    out["accuracy_sample"] = f"{len(idx)} circuits (every {max(1, n // 64)}th), complex128 batch as reference"
    # per-circuit loop of the plain path (reference-facing module), on a sample
    idx = list(range(0, n, max(1, n // 32)))
    plain = [(wl[i][0], packed_to_ops(wl[i][1]), wl[i][2]) for i in idx]
    plain_circuit_gradient(m, "64", device, *plain[0])
    torch.cuda.synchronize(device)
    t = time.perf_counter()
    for nq, ops, words in plain:
        plain_circuit_gradient(m, "64", device, nq, ops, words)
    torch.cuda.synchronize(device)
    dt = time.perf_counter() - t
    frac = work[idx].sum() / work.sum()
    out["plain_loop"] = {"sample": f"{len(idx)} circuits (every {max(1, n // 32)}th), LightningKokkos_C64 + "
                                   "AdjointJacobianKokkos_C64 per circuit",
                         "seconds": dt, "extrapolated_seconds_full_batch": dt / frac,
                         "circuits_per_s": n / (dt / frac)}
    out["speedup_vs_plain_loop"] = (dt / frac) / (ms / 1e3)
    return out


def run_batch_cpu(args):
    """The oracle (CPU restatement, OpenMP on every host core) on a sample of
    the batch: forward, <H>, adjoint Jacobian per circuit."""
    import oracle as O
    from pennylane_lightning_kokkos.circuits import batch_workload_packed, packed_to_ops

    threads = os.cpu_count() or 1
    O.set_num_threads(threads)
    n = args.batch_circuits
    wl = batch_workload_packed(n, seed=5)
    work = np.array([len(pk["gates"]) * float(1 << nq) for nq, pk, _ in wl])
    idx = list(range(0, n, max(1, n // 8)))
    letters = {"X": "PauliX", "Y": "PauliY", "Z": "PauliZ"}
    t = time.perf_counter()
    for i in idx:
        nq, pk, words = wl[i]
        ops = packed_to_ops(pk)
        psi = O.run_ops(O.zero_state(nq), ops)
        obs = ("hamiltonian", [c for c, _, _ in words],
               [("tensor", [("named", letters[x], [wi]) for wi, x in zip(w, l)]) for _, w, l in words])
        O.expval_observable(psi, obs)
        O.adjoint_jacobian(psi, [obs], ops, list(range(sum(1 for o in ops if o[3]))))
    dt = time.perf_counter() - t
    frac = work[idx].sum() / work.sum()
    return {"circuits_per_s": n / (dt / frac), "cores": threads, "kind": "port",
            "sample": f"{len(idx)} circuits (every {max(1, n // 8)}th), {dt:.1f} s, extrapolated by gate work"}


# ----------------------------------------------------------- plain 20q C1 --
def run_plain20(args, device, torch):
    """Plain method, 20 qubits complex128: 10 layers of RX, RY, RZ on every wire
    + CNOT ring (600 parameters, 800 ops), <PauliZ> on every wire and the
    20 x 600 adjoint Jacobian, through the reference-facing module; the oracle
    runs the same circuit on the host cores."""
    import oracle as O
    import pennylane_lightning_kokkos.lightning_kokkos_qubit_ops as m
    from pennylane_lightning_kokkos.circuits import hardware_efficient_ansatz

    nq = 20
    ops = hardware_efficient_ansatz(nq, 10, seed=1, rotations=("RX", "RY", "RZ"), entangler="ring")
    npar = sum(1 for o in ops if o[3])
    names, wires, invs, prms = [o[0] for o in ops], [o[1] for o in ops], [o[2] for o in ops], [o[3] for o in ops]

    def gpu():
        sv = m.LightningKokkos_C128(nq, m.InitializationSettings().set_device_id(device))
        sv.apply(names, wires, invs, prms)
        ev = np.array([sv.ExpectationValue("PauliZ", [w], [], np.array([], np.complex128)) for w in range(nq)])
        adj = m.AdjointJacobianKokkos_C128()
        tape = adj.create_ops_list(names, [np.array(p, dtype=np.float64) for p in prms], wires, invs,
                                   [np.array([], dtype=np.complex128)] * len(ops))
        obs = [m.NamedObsKokkos_C128("PauliZ", [w]) for w in range(nq)]
        jac = np.asarray(adj.adjoint_jacobian(sv, obs, tape, list(range(npar))))
        return ev, jac

    gpu()
    torch.cuda.synchronize(device)
    ts = []
    for _ in range(3):
        t = time.perf_counter()
        ev, jac = gpu()
        ts.append(time.perf_counter() - t)
    threads = os.cpu_count() or 1
    O.set_num_threads(threads)
    t = time.perf_counter()
    psi = O.run_ops(O.zero_state(nq), ops)
    ev_o = np.array([O.expval_named(psi, "PauliZ", [w]) for w in range(nq)])
    jac_o = O.adjoint_jacobian(psi, [("named", "PauliZ", [w]) for w in range(nq)], ops, list(range(npar)))
    cpu_s = time.perf_counter() - t
    return {"qubits": nq, "dtype": "complex128", "ops": len(ops), "params": npar, "observables": nq,
            "gpu_seconds_per_circuit": statistics.median(ts),
            "cpu_oracle_seconds_per_circuit": cpu_s, "cpu_cores": threads,
            "speedup_vs_cpu_oracle": cpu_s / statistics.median(ts),
            "max_abs_expval_diff_vs_oracle": float(np.max(np.abs(ev - ev_o))),
            "max_abs_jac_diff_vs_oracle": float(np.max(np.abs(jac - jac_o))),
            "api": "LightningKokkos_C128.apply / ExpectationValue / AdjointJacobianKokkos_C128.adjoint_jacobian"}


# ------------------------------------------------------- precision C3 --
def run_precision(args, device, torch):
    """Equal bytes: 32-qubit complex64 vs 31-qubit complex128 (32 GiB each),
    20 layers of RY, RZ + CNOT ladder, <H> of 200 Pauli words; the error of
    complex64 is stated against complex128 at 32 qubits (64 GiB)."""
    from pennylane_lightning_kokkos import _native as N
    from pennylane_lightning_kokkos.circuits import hardware_efficient_ansatz, random_pauli_words

    out = {}
    words = {}
    for nq in (31, 32):
        words[nq] = random_pauli_words(nq, 200, seed=3)

    def run(nq, dtype):
        ops = hardware_efficient_ansatz(nq, 20, seed=3, rotations=("RY", "RZ"), entangler="ladder")
        h = C.c_void_p()
        N.check(N.lib.plk_state_create(nq, dtype, device, C.byref(h)))
        arr = (N.PlkOp * len(ops))()
        keep = []
        for i, (name, w, inv, p) in enumerate(ops):
            wa = np.array(w, dtype=np.int64)
            pa = np.array(p or [0.0], dtype=np.float64)
            keep += [wa, pa]
            arr[i] = N.PlkOp(N.GATE_ID[name], len(w), 0, len(p), wa.ctypes.data_as(C.POINTER(C.c_int64)),
                             pa.ctypes.data_as(C.POINTER(C.c_double)), None)
        wd = words[nq]
        co = np.array([c for c, _, _ in wd])
        of = np.cumsum([0] + [len(w) for _, w, _ in wd]).astype(np.int64)
        wi = np.array([x for _, w, _ in wd for x in w], dtype=np.int64)
        le = "".join(l for _, _, l in wd).encode()
        torch.cuda.synchronize(device)
        t = time.perf_counter()
        N.check(N.lib.plk_apply_ops(h, arr, len(ops)))
        N.check(N.lib.plk_state_synchronize(h))
        t_g = time.perf_counter() - t
        v = C.c_double()
        t = time.perf_counter()
        N.check(N.lib.plk_expval_pauli_sum(h, len(co), co.ctypes.data_as(C.POINTER(C.c_double)),
                                           of.ctypes.data_as(C.POINTER(C.c_int64)),
                                           wi.ctypes.data_as(C.POINTER(C.c_int64)), le, C.byref(v)))
        t_e = time.perf_counter() - t
        return h, len(ops), t_g, t_e, v.value

    res = {}
    for nq, dt, name in ((32, N.PLK_C64, "c64_32q"), (31, N.PLK_C128, "c128_31q")):
        h, nops, t_g, t_e, val = run(nq, dt)
        ops = hardware_efficient_ansatz(nq, 20, seed=3, rotations=("RY", "RZ"), entangler="ladder")
        touched = sum(0.5 if o[0] == "CNOT" else 1.0 for o in ops)  # CNOT moves half of the amplitudes
        nbytes = 2 * (1 << nq) * (8 if dt == N.PLK_C64 else 16) * touched
        res[name] = {"gates": nops, "gates_seconds": t_g, "gates_GBps_algorithmic": nbytes / t_g / 1e9,
                     "expval_seconds": t_e, "expval": val}
        N.lib.plk_state_destroy(h)
    # error of complex64 at 32 qubits against complex128 at 32 qubits
    h64, _, _, _, v64 = run(32, N.PLK_C64)
    h128, _, _, _, v128 = run(32, N.PLK_C128)
    p64, p128 = C.c_void_p(), C.c_void_p()
    nq_, dt_ = C.c_int(), C.c_int()
    N.check(N.lib.plk_state_get(h64, C.byref(nq_), C.byref(dt_), C.byref(p64)))
    N.check(N.lib.plk_state_get(h128, C.byref(nq_), C.byref(dt_), C.byref(p128)))
    n = 1 << 32
    chunk = 1 << 28
    maxd = 0.0

    class _Arr:
        def __init__(self, ptr, shape, typestr):
            self.__cuda_array_interface__ = {"data": (ptr, False), "shape": shape, "typestr": typestr, "version": 3}

    for off in range(0, n, chunk):
        a = torch.as_tensor(_Arr(p64.value + off * 8, (chunk,), "<c8"), device=f"cuda:{device}")
        b = torch.as_tensor(_Arr(p128.value + off * 16, (chunk,), "<c16"), device=f"cuda:{device}")
        maxd = max(maxd, float((a.to(torch.complex128) - b).abs().max()))
    N.lib.plk_state_destroy(h64)
    N.lib.plk_state_destroy(h128)
    res["error_c64_vs_c128_32q"] = {"expval_abs": abs(v64 - v128), "state_max_abs": maxd,
                                     "expval_c128": v128,
                                     "reference": "complex128 GPU path at 32 qubits (parity-checked against the "
                                                  "FP64 oracle at <= 26 qubits)"}
    res["equal_bytes_speed_ratio_gates"] = res["c128_31q"]["gates_seconds"] / res["c64_32q"]["gates_seconds"]
    out.update(res)
    return out


# ---------------------------------------------------------- kernel census --
def run_kernels(args, device, torch):
    """One call of every C-ABI entry point family on a state larger than L2
    (default 26 qubits: 1 GiB complex128, 512 MiB complex64), timed with CUDA
    events on the state's stream (median of ``--census-reps``).  Each line
    gives the algorithmic bytes of the call (the state passes the operation
    needs at minimum) and the achieved GB/s; calls that return host arrays
    (probs, CDF, samples) include their device-to-host copy in the time."""
    from pennylane_lightning_kokkos import _native as N
    from pennylane_lightning_kokkos.circuits import random_pauli_words

    nq, reps = args.census_nq, max(1, args.census_reps)
    n = 1 << nq
    rng = np.random.default_rng(7)
    stream = torch.cuda.Stream(device=device)
    i64 = lambda a: np.ascontiguousarray(a, dtype=np.int64)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    P64 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))
    PD = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))

    def haar(k):
        z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        q, r = np.linalg.qr(z)
        return np.ascontiguousarray(q * (np.diag(r) / np.abs(np.diag(r))), dtype=np.complex128)

    words = random_pauli_words(nq, 20, seed=7)
    co = f64([c for c, _, _ in words])
    of = i64(np.cumsum([0] + [len(w) for _, w, _ in words]))
    wi = i64([x for _, w, _ in words for x in w])
    le = "".join(l for _, _, l in words).encode()

    def xmask(w, l):
        return sum(1 << (nq - 1 - x) for x, c in zip(w, l) if c in "XY")

    npass_words = len({xmask(w, l) for _, w, l in words})
    m3, m2, m5, m6 = haar(3), haar(2), haar(5), haar(6)
    u = f64(rng.random(1 << 20))
    shots_out = np.empty((1 << 20) * nq, dtype=np.int64)
    probs_full = np.empty(n, dtype=np.float64)
    probs_m = np.empty(1 << 14, dtype=np.float64)
    wm = i64(rng.permutation(nq)[:14])

    out = {"qubits": nq, "reps": reps, "timing": "CUDA events on the state's stream, median of reps",
           "calls": {}}
    for dtype, dname, sz in ((N.PLK_C128, "c128", 16), (N.PLK_C64, "c64", 8)):
        S = n * sz
        hs = []
        for _ in range(2):
            h = C.c_void_p()
            N.check(N.lib.plk_state_create(nq, dtype, device, C.byref(h)))
            N.check(N.lib.plk_state_set_stream(h, C.c_void_p(stream.cuda_stream)))
            hs.append(h)
        a, b = hs
        hw = i64([0])
        for w in range(nq):
            hw[0] = w
            N.check(N.lib.plk_apply_gate(a, N.GATE_ID["Hadamard"], P64(hw), 1, 0, None, 0))
        N.check(N.lib.plk_state_copy(b, a))
        keep = []

        def gate(name, wires, params=()):
            w, p = i64(wires), f64(list(params) or [0.0])
            keep.extend([w, p])
            g = N.GATE_ID[name]
            return lambda: N.check(N.lib.plk_apply_gate(a, g, P64(w), len(w), 0, PD(p), len(params)))

        def matrix(m, wires):
            w = i64(wires)
            keep.extend([w, m])
            return lambda: N.check(N.lib.plk_apply_matrix(a, m.ctypes.data_as(C.POINTER(C.c_double)), P64(w),
                                                          len(w), 0))

        sc, v, vr, vi = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        dptr, nq_, dt_ = C.c_void_p(), C.c_int(), C.c_int()
        N.check(N.lib.plk_state_get(a, C.byref(nq_), C.byref(dt_), C.byref(dptr)))
        dout = torch.zeros(16, dtype=torch.float64, device=f"cuda:{device}")
        dout_p = C.cast(C.c_void_p(dout.data_ptr()), C.POINTER(C.c_double))
        w16 = i64(list(range(15)) + [-1])
        sp = C.c_void_p(stream.cuda_stream)
        zb = np.array([N.GATE_ID["PauliZ"]] * 20, dtype=np.int32)
        zw = i64(range(20))
        lo, mid, hi = nq - 3, nq // 2, 1  # wire -> rev bit: 2, ~n/2, n-2
        calls = [
            ("reset (|0>)", lambda: N.check(N.lib.plk_state_reset(a)), S),
            ("PauliX low wire", gate("PauliX", [lo]), 2 * S),
            ("PauliX high wire", gate("PauliX", [hi]), 2 * S),
            ("Hadamard", gate("Hadamard", [mid]), 2 * S),
            ("RX", gate("RX", [mid], [0.3]), 2 * S),
            ("CNOT", gate("CNOT", [hi, lo]), S),
            ("CRY", gate("CRY", [lo, mid], [0.4]), S),
            ("IsingXX", gate("IsingXX", [mid, hi], [0.5]), 2 * S),
            ("SingleExcitation", gate("SingleExcitation", [lo, hi], [0.6]), S),
            ("DoubleExcitation", gate("DoubleExcitation", [0, 5, 9, lo], [0.7]), S // 4),
            ("Toffoli", gate("Toffoli", [hi, mid, lo]), S // 2),
            ("CSWAP", gate("CSWAP", [hi, mid, lo]), S // 2),
            ("MultiRZ (5 wires)", gate("MultiRZ", [0, 3, mid, lo, nq - 1], [0.8]), 2 * S),
            ("Haar 2-qubit matrix", matrix(m2, [mid, lo]), 2 * S),
            ("Haar 3-qubit matrix", matrix(m3, [hi, mid, lo]), 2 * S),
            ("Haar 5-qubit matrix", matrix(m5, [hi, 4, mid, lo, nq - 1]), 2 * S),
            ("Haar 6-qubit matrix", matrix(m6, [hi, 4, 7, mid, lo, nq - 1]), 2 * S),
            ("Haar 6-qubit matrix, CUDA cores", lambda: (N.check(N.lib.plk_set_dense_tensor_cores(0)),
                                                         matrix(m6, [hi, 4, 7, mid, lo, nq - 1])(),
                                                         N.check(N.lib.plk_set_dense_tensor_cores(1))), 2 * S),
            ("generator IsingXX", lambda: N.check(N.lib.plk_apply_generator(a, N.GATE_ID["IsingXX"], P64(zw), 2, 0,
                                                                            C.byref(sc))), 2 * S),
            ("expval PauliZ", lambda: N.check(N.lib.plk_expval_named(a, N.GATE_ID["PauliZ"], P64(zw), 1,
                                                                     C.byref(v))), S),
            ("expval PauliX", lambda: N.check(N.lib.plk_expval_named(a, N.GATE_ID["PauliX"], P64(zw), 1,
                                                                     C.byref(v))), S),
            ("expval 20 x PauliZ (one pass)", lambda: N.check(N.lib.plk_expval_named_batch(
                a, 20, zb.ctypes.data_as(C.POINTER(C.c_int32)), P64(zw), PD(probs_m))), S),
            ("expval PauliZ, allocation-free entry", lambda: N.check(N.lib.plk_expval_pauliz_noalloc(
                dptr, nq, dtype, 1, P64(w16), dout_p, sp)), S),
            ("expval 16 x PauliZ, allocation-free entry", lambda: N.check(N.lib.plk_expval_pauliz_noalloc(
                dptr, nq, dtype, 16, P64(w16), dout_p, sp)), S),
            ("expval 2-qubit matrix", lambda: N.check(N.lib.plk_expval_matrix(
                a, m2.ctypes.data_as(C.POINTER(C.c_double)), P64(i64([mid, lo])), 2, C.byref(v))), S),
            ("expval 3-qubit matrix", lambda: N.check(N.lib.plk_expval_matrix(
                a, m3.ctypes.data_as(C.POINTER(C.c_double)), P64(i64([hi, mid, lo])), 3, C.byref(v))), S),
            (f"expval 20 Pauli words ({npass_words} passes)", lambda: N.check(N.lib.plk_expval_pauli_sum(
                a, len(co), PD(co), P64(of), P64(wi), le, C.byref(v))), npass_words * S),
            (f"apply 20 Pauli words (H|psi>, {npass_words} gathers)", lambda: N.check(N.lib.plk_apply_pauli_sum(
                b, a, len(co), PD(co), P64(of), P64(wi), le)), (npass_words + 1) * S),
            ("inner product", lambda: N.check(N.lib.plk_inner_product(a, b, C.byref(vr), C.byref(vi))), 2 * S),
            ("axpy", lambda: N.check(N.lib.plk_state_axpy(b, 0.5, 0.25, a)), 3 * S),
            ("copy", lambda: N.check(N.lib.plk_state_copy(b, a)), 2 * S),
            ("probs() to host", lambda: N.check(N.lib.plk_probs(a, None, 0, PD(probs_full))), S + n * 8),
            ("probs(14 wires) to host", lambda: N.check(N.lib.plk_probs(a, P64(wm), 14, PD(probs_m))), S),
            ("CDF to host", lambda: N.check(N.lib.plk_cdf(a, PD(probs_full))), 2 * S + n * 8),
            ("sample 2^20 shots from uniforms", lambda: N.check(N.lib.plk_sample_from_uniforms(
                a, PD(u), len(u), P64(shots_out))), 2 * S),
        ]
        res = {}
        for name, fn, nbytes in calls:
            fn()  # warm-up
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize(device)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize(device)
                ts.append(e0.elapsed_time(e1))
            ms = statistics.median(ts)
            res[name] = {"ms": ms, "algorithmic_bytes": nbytes, "GBps": nbytes / (ms * 1e6)}
        for h in hs:
            N.lib.plk_state_destroy(h)
        out["calls"][dname] = res
    return out


# ------------------------------------------------------------- replicas --
def aggregate_ranks(dist, torch, ms, nbytes, device="cpu"):
    """Whole-job figures of independent replicas: the slowest rank's time and
    the bytes of all ranks (value = all ranks' bytes / max time)."""
    t = torch.tensor([ms, nbytes], dtype=torch.float64, device=device)
    mx = t.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    sm = t.clone()
    dist.all_reduce(sm, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(sm[1])


# ------------------------------------------------------------------ main --
def main(argv=None):
    args = parse_args(argv)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        res = run_reference_arm(args, rank)
        if res is not None:
            print(json.dumps(res), flush=True)
        return 0

    import torch

    device = local_rank
    torch.cuda.set_device(device)
    if args.only:
        if rank == 0:
            fn = {"adjoint": run_adjoint, "batch": run_batch, "plain20": run_plain20, "precision": run_precision,
                  "kernels": run_kernels, "parity": run_parity}
            print(json.dumps({args.only: fn[args.only](args, device, torch)}), flush=True)
        return 0
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", device))

    def barrier():
        if dist is not None:
            dist.barrier()

    sweep = run_device_sweep(args, device, torch, barrier)
    total_ms = sweep["total_ms"]
    total_bytes = sweep["total_bytes"]
    if dist is not None:
        total_ms, total_bytes = aggregate_ranks(dist, torch, total_ms, total_bytes, f"cuda:{device}")
    value = total_bytes / (total_ms * 1e6)

    peak, peak_kind = peaks()
    shares = {g: ms / sweep["total_ms"] for g, ms in sweep["per_gate_ms"].items()}
    per_gate = {g: {"GBps": sweep["bytes_per_gate"][g] / (ms * 1e6), "share": shares[g],
                    "ms_per_app": ms / (args.steps * sum(1 for a in sweep["plan"] if a["name"] == g))}
                for g, ms in sweep["per_gate_ms"].items()}
    dom = max(shares, key=shares.get)
    n_apps_dom = sum(1 for a in sweep["plan"] if a["name"] == dom) * args.steps
    roof = {"bound": "hbm", "kernel": f"{dom} gate kernel",
            "achieved": per_gate[dom]["GBps"], "peak": peak, "unit": "GB/s",
            "frac": per_gate[dom]["GBps"] / peak, "peak_kind": peak_kind,
            "traffic": None, "launches": n_apps_dom,
            "overall_frac": value / (peak * world)}
    if dom in KERNEL_LIMITS:
        roof["limit"] = KERNEL_LIMITS[dom]
    prof = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(prof):
        try:
            tr = json.load(open(prof)).get(dom)
            if tr:
                roof["traffic"] = tr
        except Exception:
            pass

    from pennylane_lightning_kokkos import _native as N

    dtype = ("complex128 storage, double-float arithmetic (FP32 pipe)" if N.c128_arithmetic() == "double-float"
             else "complex128 (native FP64 arithmetic)")
    result = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded gate sweep, seed 2)",
        "config": sweep_config(args),
        "step_plan": f"{len(sweep['plan'])} applications: {args.reps} per gate type and wire range, the same every "
                     "step",
        "parallelism": f"replicas x{world}",
        "roofline": roof, "per_gate": per_gate, "per_range": sweep["per_range"], "clocks": sweep["clocks"],
        "gpu_launches": sweep["launches"],
    }
    if sweep["fp64"]:
        result["per_gate_fp64"] = sweep["fp64"]
    if rank == 0 and not args.no_e2e:
        result["e2e"] = run_e2e(args, device, torch, sweep["plan"], steps=max(1, min(args.steps, 3)))
    if rank == 0 and not args.no_adjoint:
        try:
            result["adjoint_26q"] = run_adjoint(args, device, torch)
        except Exception as e:  # report, do not hide the main number
            result["adjoint_26q"] = {"error": repr(e)}
    if rank == 0 and not args.no_batch:
        try:
            result["batch"] = run_batch(args, device, torch)
        except Exception as e:
            result["batch"] = {"error": repr(e)}
    if rank == 0 and not args.no_plain20:
        try:
            result["plain_20q"] = run_plain20(args, device, torch)
        except Exception as e:
            result["plain_20q"] = {"error": repr(e)}
    if rank == 0 and not args.no_precision:
        try:
            result["precision"] = run_precision(args, device, torch)
        except Exception as e:
            result["precision"] = {"error": repr(e)}
    if rank == 0 and not args.no_cpu:
        result["cpu_baseline"], sv_ref, plan_ref = run_cpu_baseline(args)
        parity = {}
        try:
            parity["sweep_state"] = sweep_parity(args, device, sv_ref, plan_ref)
        except Exception as e:
            parity["sweep_state"] = {"error": repr(e)}
        del sv_ref
        if not args.no_adjoint:
            try:
                parity["adjoint_26q"] = run_adjoint_parity(args, device, torch, args.parity_layers or 2)
            except Exception as e:
                parity["adjoint_26q"] = {"error": repr(e)}
        if "error" not in result.get("plain_20q", {"error": 1}):
            p20 = result["plain_20q"]
            parity["plain_20q"] = {k: p20[k] for k in ("max_abs_expval_diff_vs_oracle", "max_abs_jac_diff_vs_oracle")}
        parity["full_size"] = ("bench.py --only parity: 26-qubit 40-layer gradients, 31/32-qubit short circuits; "
                               "record in profiles/parity_full_size.md")
        result["parity"] = parity
        if not args.no_batch and "error" not in result.get("batch", {}):
            try:
                result["batch"]["cpu_oracle"] = run_batch_cpu(args)
                result["batch"]["speedup_vs_cpu_oracle"] = (result["batch"]["circuits_per_s"]
                                                            / result["batch"]["cpu_oracle"]["circuits_per_s"])
            except Exception as e:
                result["batch"]["cpu_oracle"] = {"error": repr(e)}
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(result), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
