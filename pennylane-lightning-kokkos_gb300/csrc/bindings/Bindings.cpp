// Bindings.cpp — the `lightning_kokkos_qubit_ops` Python module.
//
// Keeps the class and method surface of the reference's pybind11 module
// (bindings/Bindings.cpp:50-968): LightningKokkos_C64/C128 with one method
// per gate, apply / applyGenerator / ExpectationValue / probs /
// GenerateSamples / DeviceToHost / HostToDevice / setBasisState /
// setStateVector / numQubits / dataLength / resetKokkos; the observable
// classes; OpsStructKokkos and AdjointJacobianKokkos; InitializationSettings
// and the module functions; the PLException error type.  Underneath, the
// calls go to the C++ host layer in ../host, which drives the sm_103a
// kernels through include/plk_gb300.h.
#include <pybind11/complex.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <sstream>

#include "../host/AdjointGB.hpp"

namespace py = pybind11;
using namespace Pennylane::LightningGB300;

namespace {

template <class T> std::vector<std::complex<T>> to_cvec(const py::array_t<std::complex<T>, py::array::c_style | py::array::forcecast> &a) {
    const auto b = a.request();
    const auto *p = static_cast<const std::complex<T> *>(b.ptr);
    return std::vector<std::complex<T>>(p, p + b.size);
}

// the named gates exposed as methods (Bindings.cpp:87-360)
const char *kGateMethods[] = {"PauliX", "PauliY", "PauliZ", "Hadamard", "S", "T", "CNOT", "SWAP", "CSWAP",
                              "Toffoli", "CY", "CZ", "PhaseShift", "ControlledPhaseShift", "RX", "RY", "RZ",
                              "Rot", "CRX", "CRY", "CRZ", "CRot", "IsingXX", "IsingXY", "IsingYY", "IsingZZ",
                              "MultiRZ", "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus",
                              "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus"};

std::string device_config_text(int device) {
    plk_device_info info;
    std::ostringstream ss;
    if (plk_get_device_info(device, &info) != PLK_OK) {
        ss << "GB300 core: no CUDA device (" << plk_last_error() << ")\n";
        return ss.str();
    }
    ss << "GB300 core " << plk_version() << "\n"
       << "  Device: " << info.name << " (sm_" << info.cc_major << info.cc_minor << ")\n"
       << "  SMs: " << info.sm_count << "\n"
       << "  HBM: " << info.total_mem / (1024 * 1024) << " MiB total, " << info.free_mem / (1024 * 1024)
       << " MiB free\n"
       << "  SM clock: " << info.clock_khz / 1000 << " MHz, memory clock: " << info.mem_clock_khz / 1000
       << " MHz, bus width: " << info.mem_bus_width << " bit\n";
    return ss.str();
}

py::dict device_config_dict(int device) {
    using namespace py::literals;
    py::dict d;
    plk_device_info info;
    if (plk_get_device_info(device, &info) != PLK_OK) {
        d["Backend"] = py::dict("available"_a = false, "error"_a = std::string(plk_last_error()));
        return d;
    }
    d["Backend"] = py::dict("Parallel"_a = "CUDA (sm_103a kernels)", "available"_a = true);
    d["Device"] = py::dict("name"_a = std::string(info.name), "sm_count"_a = info.sm_count,
                           "compute_capability"_a = std::to_string(info.cc_major) + "." + std::to_string(info.cc_minor),
                           "total_mem"_a = info.total_mem, "free_mem"_a = info.free_mem,
                           "sm_clock_khz"_a = info.clock_khz, "mem_clock_khz"_a = info.mem_clock_khz,
                           "mem_bus_width"_a = info.mem_bus_width);
    return d;
}

template <class PrecisionT, class ParamT> void bind_precision(py::module_ &m) {
    using SV = StateVectorGB<PrecisionT>;
    using np_arr_r = py::array_t<ParamT, py::array::c_style | py::array::forcecast>;
    using np_arr_c = py::array_t<std::complex<ParamT>, py::array::c_style | py::array::forcecast>;
    const std::string bits = std::to_string(sizeof(std::complex<PrecisionT>) * 8);

    auto cls = py::class_<SV>(m, ("LightningKokkos_C" + bits).c_str());
    cls.def(py::init([](size_t n) { return new SV(n); }))
        .def(py::init([](size_t n, const InitializationSettings &a) { return new SV(n, a); }))
        .def(py::init([](const np_arr_c &arr) {
            auto b = arr.request();
            return new SV(static_cast<const std::complex<PrecisionT> *>(b.ptr), (size_t)arr.size());
        }))
        .def(py::init([](const np_arr_c &arr, const InitializationSettings &a) {
            auto b = arr.request();
            return new SV(static_cast<const std::complex<PrecisionT> *>(b.ptr), (size_t)arr.size(), a);
        }))
        .def("setBasisState", [](SV &sv, size_t index) { sv.setBasisState(index); }, "Create Basis State on Device.")
        .def(
            "setStateVector",
            [](SV &sv, const std::vector<size_t> &indices, const np_arr_c &state) {
                sv.setStateVector(indices, to_cvec<ParamT>(state));
            },
            "Set State Vector on device with values and their corresponding indices")
        .def(
            "Identity", [](SV &, const std::vector<size_t> &, bool, const std::vector<ParamT> &) {},
            "Apply the Identity gate.");
    for (const char *name : kGateMethods) {
        const int g = gate_id(name);
        cls.def(
            name,
            [g](SV &sv, const std::vector<size_t> &wires, bool adjoint, const std::vector<ParamT> &params) {
                sv.applyGate(g, wires, adjoint, std::vector<PrecisionT>(params.begin(), params.end()));
            },
            (std::string("Apply the ") + name + " gate.").c_str());
    }
    cls.def("apply",
            [](SV &sv, const std::vector<std::string> &names, const std::vector<std::vector<size_t>> &wires,
               const std::vector<bool> &adj, const std::vector<std::vector<PrecisionT>> &params) {
                sv.applyOperation(names, wires, adj, params);
            })
        .def("apply",
             [](SV &sv, const std::vector<std::string> &names, const std::vector<std::vector<size_t>> &wires,
                const std::vector<bool> &adj) { sv.applyOperation(names, wires, adj); })
        .def(
            "apply",
            [](SV &sv, const std::string &name, const std::vector<size_t> &wires, bool inv,
               const std::vector<std::vector<ParamT>> & /*params*/, const np_arr_c &matrix) {
                sv.applyOperation(name, wires, inv, std::vector<PrecisionT>{}, to_cvec<ParamT>(matrix));
            },
            "Apply operation via the gate matrix")
        .def(
            "applyGenerator",
            [](SV &sv, const std::string &name, const std::vector<size_t> &wires, bool adj,
               const std::vector<PrecisionT> &params) { return sv.applyGenerator(name, wires, adj, params); })
        .def(
            "ExpectationValue",
            [](SV &sv, const std::string &name, const std::vector<size_t> &wires, const std::vector<ParamT> &params,
               const np_arr_c &matrix) {
                return (PrecisionT)MeasuresGB<PrecisionT>(sv).getExpectationValue(
                    name, wires, std::vector<PrecisionT>(params.begin(), params.end()), to_cvec<ParamT>(matrix));
            },
            "Calculate the expectation value of the given observable.")
        .def(
            "ExpectationValue",
            [](SV &sv, const std::vector<std::string> &names, const std::vector<size_t> &wires,
               const std::vector<std::vector<ParamT>> & /*params*/, const np_arr_c &matrix) {
                std::string concat = "#";
                for (const auto &s : names) concat += s;
                return (PrecisionT)MeasuresGB<PrecisionT>(sv).getExpectationValue(concat, wires, {},
                                                                                  to_cvec<ParamT>(matrix));
            },
            "Calculate the expectation value of the given observable.")
        .def(
            "ExpectationValue",
            [](SV &sv, const std::vector<size_t> &wires, const np_arr_c &matrix) {
                return (PrecisionT)MeasuresGB<PrecisionT>(sv).getExpectationValue(wires, to_cvec<ParamT>(matrix));
            },
            "Calculate the expectation value of the given observable.")
        .def(
            "ExpectationValue",
            [](SV &sv, const np_arr_c &data, const std::vector<size_t> &indices, const std::vector<size_t> &indptr) {
                return (PrecisionT)MeasuresGB<PrecisionT>(sv).getExpectationValue(to_cvec<ParamT>(data), indices,
                                                                                  indptr);
            },
            "Calculate the expectation value of the given observable.")
        .def("probs",
             [](SV &sv, const std::vector<size_t> &wires) {
                 auto p = MeasuresGB<PrecisionT>(sv).probs(wires);
                 py::array_t<ParamT> out(p.size());
                 auto *o = out.mutable_data();
                 for (size_t i = 0; i < p.size(); i++) o[i] = (ParamT)p[i];
                 return out;
             })
        .def("GenerateSamples",
             [](SV &sv, size_t num_wires, size_t num_shots) {
                 auto r = MeasuresGB<PrecisionT>(sv).generate_samples(num_shots);
                 py::array_t<size_t> out({num_shots, num_wires});
                 auto *o = out.mutable_data();
                 for (size_t i = 0; i < r.size(); i++) o[i] = (size_t)r[i];
                 return out;
             })
        .def(
            "DeviceToHost",
            [](SV &sv, py::array_t<std::complex<PrecisionT>, py::array::c_style> &host) {
                if (host.size()) sv.DeviceToHost(host.mutable_data(), (size_t)host.size());
            },
            "Synchronize data from the GPU device to host.")
        .def(
            "HostToDevice",
            [](SV &sv, const np_arr_c &host) {
                auto b = host.request();
                const size_t length = (size_t)b.shape[0];
                if (length) sv.HostToDevice(static_cast<const std::complex<PrecisionT> *>(b.ptr), length);
            },
            "Synchronize data from the host device to GPU.")
        .def("numQubits", &SV::getNumQubits)
        .def("dataLength", &SV::getLength)
        .def("resetKokkos", &SV::resetStateVector)
        // GB300 additions: raw device pointer (for zero-copy interop), queued
        // host copies and the stream they go on, and the Pauli-sum
        // expectation value
        .def("device_ptr", [](SV &sv) { return (uintptr_t)sv.devicePtr(); })
        .def(
            "HostToDeviceAsync",
            [](SV &sv, py::array_t<std::complex<PrecisionT>, py::array::c_style> &host) {
                if (host.size()) sv.HostToDeviceAsync(host.data(), (size_t)host.size());
            },
            py::arg("host").noconvert(),
            "Queue the host-to-device copy on the state's stream and return; the array (of the state's dtype: no "
            "conversion copy is made) must stay alive and unchanged until synchronize().")
        .def(
            "DeviceToHostAsync",
            [](SV &sv, py::array_t<std::complex<PrecisionT>, py::array::c_style> &host) {
                if (host.size()) sv.DeviceToHostAsync(host.mutable_data(), (size_t)host.size());
            },
            py::arg("host").noconvert(),
            "Queue the device-to-host copy on the state's stream and return; read the array after synchronize().")
        .def(
            "set_stream", [](SV &sv, uintptr_t stream) { sv.setStream((void *)stream); },
            "Queue this state's work on a CUDA stream (an address such as torch.cuda.Stream().cuda_stream; 0: the "
            "library's stream).")
        .def("synchronize", [](SV &sv) { sv.synchronize(); }, "Wait for this state's queued work.")
        .def("ExpectationValuePauliSum",
             [](SV &sv, const std::vector<double> &coeffs, const std::vector<std::vector<size_t>> &wires,
                const std::vector<std::string> &letters) {
                 if (coeffs.size() != wires.size() || coeffs.size() != letters.size())
                     pl_abort("coefficients, wires and Pauli strings differ in length");
                 std::vector<PauliWord> words;
                 for (size_t t = 0; t < coeffs.size(); t++) {
                     if (wires[t].size() != letters[t].size()) pl_abort("Pauli string length != wire count");
                     words.push_back({coeffs[t], wires[t], letters[t]});
                 }
                 return MeasuresGB<PrecisionT>(sv).pauliSum(words);
             });

    // ---- observables (Bindings.cpp:591-736) ----
    using Obs = ObservableGB<PrecisionT>;
    py::class_<Obs, std::shared_ptr<Obs>>(m, ("ObservableKokkos_C" + bits).c_str(), py::module_local());

    using Named = NamedObsGB<PrecisionT>;
    py::class_<Named, std::shared_ptr<Named>, Obs>(m, ("NamedObsKokkos_C" + bits).c_str(), py::module_local())
        .def(py::init([](const std::string &name, const std::vector<size_t> &wires) { return Named(name, wires); }))
        .def("__repr__", &Named::getObsName)
        .def("get_wires", &Named::getWires, "Get wires of observables")
        .def("__eq__", [](const Named &self, py::handle other) -> bool {
            if (!py::isinstance<Named>(other)) return false;
            return self == other.cast<Named>();
        });

    using Herm = HermitianObsGB<PrecisionT>;
    py::class_<Herm, std::shared_ptr<Herm>, Obs>(m, ("HermitianObsKokkos_C" + bits).c_str(), py::module_local())
        .def(py::init([](const np_arr_c &matrix, const std::vector<size_t> &wires) {
            return Herm(to_cvec<ParamT>(matrix), wires);
        }))
        .def("__repr__", &Herm::getObsName)
        .def("get_wires", &Herm::getWires, "Get wires of observables")
        .def("__eq__", [](const Herm &self, py::handle other) -> bool {
            if (!py::isinstance<Herm>(other)) return false;
            return self == other.cast<Herm>();
        });

    using Tensor = TensorProdObsGB<PrecisionT>;
    py::class_<Tensor, std::shared_ptr<Tensor>, Obs>(m, ("TensorProdObsKokkos_C" + bits).c_str(), py::module_local())
        .def(py::init([](const std::vector<std::shared_ptr<Obs>> &obs) { return Tensor(obs); }))
        .def("__repr__", &Tensor::getObsName)
        .def("get_wires", &Tensor::getWires, "Get wires of observables")
        .def("__eq__", [](const Tensor &self, py::handle other) -> bool {
            if (!py::isinstance<Tensor>(other)) return false;
            return self == other.cast<Tensor>();
        });

    using Ham = HamiltonianGB<PrecisionT>;
    py::class_<Ham, std::shared_ptr<Ham>, Obs>(m, ("HamiltonianKokkos_C" + bits).c_str(), py::module_local())
        .def(py::init([](const np_arr_r &coeffs, const std::vector<std::shared_ptr<Obs>> &obs) {
            auto b = coeffs.request();
            const auto *p = static_cast<const ParamT *>(b.ptr);
            return Ham(std::vector<PrecisionT>(p, p + b.size), obs);
        }))
        .def("__repr__", &Ham::getObsName)
        .def("get_wires", &Ham::getWires, "Get wires of observables")
        .def("__eq__", [](const Ham &self, py::handle other) -> bool {
            if (!py::isinstance<Ham>(other)) return false;
            return self == other.cast<Ham>();
        });

    using Sparse = SparseHamiltonianGB<PrecisionT>;
    py::class_<Sparse, std::shared_ptr<Sparse>, Obs>(m, ("SparseHamiltonianKokkos_C" + bits).c_str(),
                                                     py::module_local())
        .def(py::init([](const np_arr_c &data, const std::vector<size_t> &indices, const std::vector<size_t> &indptr,
                         const std::vector<size_t> &wires) {
            return Sparse(to_cvec<ParamT>(data), indices, indptr, wires);
        }))
        .def("__repr__", &Sparse::getObsName)
        .def("get_wires", &Sparse::getWires, "Get wires of observables")
        .def("__eq__", [](const Sparse &self, py::handle other) -> bool {
            if (!py::isinstance<Sparse>(other)) return false;
            return self == other.cast<Sparse>();
        });

    // ---- adjoint (Bindings.cpp:741-821) ----
    using Ops = OpsData<PrecisionT>;
    py::class_<Ops>(m, ("OpsStructKokkos_C" + bits).c_str(), py::module_local())
        .def(py::init<const std::vector<std::string> &, const std::vector<std::vector<PrecisionT>> &,
                      const std::vector<std::vector<size_t>> &, const std::vector<bool> &,
                      const std::vector<std::vector<std::complex<PrecisionT>>> &>())
        .def("__repr__", [](const Ops &ops) {
            std::ostringstream ss;
            for (size_t i = 0; i < ops.getSize(); i++) {
                ss << "{'name': " << ops.getOpsName()[i] << ", 'params': " << vec_str(ops.getOpsParams()[i])
                   << ", 'inv': " << ops.getOpsInverses()[i] << "}";
                if (i + 1 < ops.getSize()) ss << ",";
            }
            return "Operations: [" + ss.str() + "]";
        });

    using Adj = AdjointJacobianGB<PrecisionT>;
    py::class_<Adj>(m, ("AdjointJacobianKokkos_C" + bits).c_str(), py::module_local())
        .def(py::init<>())
        .def("create_ops_list",
             [](Adj &, const std::vector<std::string> &names, const std::vector<np_arr_r> &params,
                const std::vector<std::vector<size_t>> &wires, const std::vector<bool> &inverses,
                const std::vector<np_arr_c> &matrices) {
                 std::vector<std::vector<PrecisionT>> cp(params.size());
                 std::vector<std::vector<std::complex<PrecisionT>>> cm(matrices.size());
                 for (size_t i = 0; i < names.size(); i++) {
                     if (i < params.size()) {
                         auto b = params[i].request();
                         const auto *p = static_cast<const ParamT *>(b.ptr);
                         cp[i].assign(p, p + b.size);
                     }
                     if (i < matrices.size() && matrices[i].size()) cm[i] = to_cvec<ParamT>(matrices[i]);
                 }
                 return Ops(names, cp, wires, inverses, cm);
             })
        .def("adjoint_jacobian",
             [](Adj &adj, const SV &sv, const std::vector<std::shared_ptr<Obs>> &obs, const Ops &ops,
                const std::vector<size_t> &trainable) {
                 std::vector<double> flat;
                 adj.adjointJacobianFlat(sv, flat, obs, ops, trainable, false);
                 py::array_t<ParamT> out({obs.size(), trainable.size()});
                 auto *o = out.mutable_data();
                 for (size_t i = 0; i < flat.size(); i++) o[i] = (ParamT)flat[i];
                 return out;
             })
        .def("adjoint_jacobian",
             [](Adj &adj, const SV &sv, const std::vector<std::shared_ptr<Obs>> &obs, const Ops &ops,
                const std::vector<size_t> &trainable, bool apply_operations) {
                 std::vector<double> flat;
                 adj.adjointJacobianFlat(sv, flat, obs, ops, trainable, apply_operations);
                 py::array_t<ParamT> out({obs.size(), trainable.size()});
                 auto *o = out.mutable_data();
                 for (size_t i = 0; i < flat.size(); i++) o[i] = (ParamT)flat[i];
                 return out;
             });
}

} // namespace

PYBIND11_MODULE(lightning_kokkos_qubit_ops, m) {
    py::options options;
    options.disable_function_signatures();
    py::register_exception<LightningException>(m, "PLException");

    bind_precision<float, float>(m);
    bind_precision<double, double>(m);

    // Kokkos runtime hooks become no-ops: the CUDA context is created lazily.
    m.def("kokkos_start", []() {});
    m.def("kokkos_end", []() {});
    m.def("kokkos_config_info", []() { return device_config_dict(0); }, "Device configuration query.");
    m.def("print_configuration", []() { return device_config_text(0); }, "Device configuration query.");
    m.def("device_count", []() {
        int c = 0;
        plk_device_count(&c);
        return c;
    });

    using IS = InitializationSettings;
    auto is = py::class_<IS>(m, "InitializationSettings");
    is.def(py::init<>());
#define PLK_IS_FIELD(NAME, TYPE)                                                                                       \
    is.def("get_" #NAME, [](const IS &s) { return s.NAME; });                                                          \
    is.def("has_" #NAME, [](const IS &s) { return s.has_##NAME; });                                                    \
    is.def("set_" #NAME, [](IS &s, TYPE v) -> IS & {                                                                   \
        s.NAME = v;                                                                                                    \
        s.has_##NAME = true;                                                                                           \
        return s;                                                                                                      \
    }, py::return_value_policy::reference_internal);
    PLK_IS_FIELD(num_threads, int)
    PLK_IS_FIELD(device_id, int)
    PLK_IS_FIELD(map_device_id_by, const std::string &)
    PLK_IS_FIELD(disable_warnings, bool)
    PLK_IS_FIELD(print_configuration, bool)
    PLK_IS_FIELD(tune_internals, bool)
    PLK_IS_FIELD(tools_libs, const std::string &)
    PLK_IS_FIELD(tools_help, bool)
    PLK_IS_FIELD(tools_args, const std::string &)
#undef PLK_IS_FIELD
    is.def("__repr__", [](const IS &a) {
        std::ostringstream ss;
        ss << "InitializationSettings:\n"
           << "num_threads = " << a.num_threads << '\n'
           << "device_id = " << a.device_id << '\n'
           << "map_device_id_by = " << a.map_device_id_by << '\n'
           << "disable_warnings = " << a.disable_warnings << '\n'
           << "print_configuration = " << a.print_configuration << '\n'
           << "tune_internals = " << a.tune_internals << '\n'
           << "tools_libs = " << a.tools_libs << '\n'
           << "tools_help = " << a.tools_help << '\n'
           << "tools_args = " << a.tools_args << '\n';
        return ss.str();
    });
}
