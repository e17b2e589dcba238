// StateVectorGB.hpp — C++ host layer over the C ABI: the state vector.
//
// Mirrors StateVectorKokkos<T> (simulator/StateVectorKokkos.hpp): same
// constructors, gate dispatch by name (applyOperation :585-676), generators
// (applyGenerator :687-695), matrix application and data movers.  All device
// work goes through include/plk_gb300.h; this header has no CUDA dependency.
#pragma once

#include <complex>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "plk_gb300.h"

namespace Pennylane::LightningGB300 {

// Error convention of the reference (util/Error.hpp:27-141): failures throw
// LightningException, which the Python module maps to PLException.
class LightningException : public std::exception {
    std::string msg_;

  public:
    explicit LightningException(std::string msg) : msg_(std::move(msg)) {}
    const char *what() const noexcept override { return msg_.c_str(); }
};

[[noreturn]] inline void pl_abort(const std::string &msg) { throw LightningException(msg); }

inline void check(int status) {
    if (status != PLK_OK) throw LightningException(plk_last_error());
}

// Replacement of Kokkos::InitializationSettings (bindings/Bindings.cpp:854-967):
// the same nine fields; device_id selects the CUDA device, the others are
// kept for interface compatibility.
struct InitializationSettings {
    int num_threads = 0;
    int device_id = 0;
    std::string map_device_id_by;
    bool disable_warnings = false;
    bool print_configuration = false;
    bool tune_internals = false;
    std::string tools_libs;
    bool tools_help = false;
    std::string tools_args;
    bool has_num_threads = false, has_device_id = false, has_map_device_id_by = false, has_disable_warnings = false,
         has_print_configuration = false, has_tune_internals = false, has_tools_libs = false, has_tools_help = false,
         has_tools_args = false;
};

inline int gate_id(const std::string &name) {
    int32_t g = -1;
    if (plk_gate_from_name(name.c_str(), &g) != PLK_OK) return -1;
    return g;
}

template <class T> constexpr int dtype_of() { return std::is_same_v<T, float> ? PLK_C64 : PLK_C128; }

template <class PrecisionT> class StateVectorGB {
  public:
    using ComplexT = std::complex<PrecisionT>;

    explicit StateVectorGB(size_t num_qubits, const InitializationSettings &args = {})
        : num_qubits_(num_qubits), device_(args.device_id) {
        if (num_qubits == 0) pl_abort("a state needs at least one qubit");
        check(plk_state_create((int)num_qubits, dtype_of<PrecisionT>(), device_, &h_));
    }
    StateVectorGB(const ComplexT *host, size_t length, const InitializationSettings &args = {})
        : StateVectorGB(log2_exact(length), args) {
        HostToDevice(host, length);
    }
    StateVectorGB(const StateVectorGB &other) : num_qubits_(other.num_qubits_), device_(other.device_) {
        check(plk_state_create((int)num_qubits_, dtype_of<PrecisionT>(), device_, &h_));
        check(plk_state_copy(h_, other.h_));
    }
    StateVectorGB &operator=(const StateVectorGB &) = delete;
    ~StateVectorGB() {
        if (h_) plk_state_destroy(h_);
    }

    static size_t log2_exact(size_t length) {
        size_t n = 0;
        while ((size_t(1) << n) < length) n++;
        if ((size_t(1) << n) != length || n == 0) pl_abort("state length must be a power of two (>= 2)");
        return n;
    }

    [[nodiscard]] plk_state handle() const { return h_; }
    [[nodiscard]] size_t getNumQubits() const { return num_qubits_; }
    [[nodiscard]] size_t getLength() const { return size_t(1) << num_qubits_; }
    [[nodiscard]] int device() const { return device_; }
    [[nodiscard]] void *devicePtr() const {
        void *p = nullptr;
        check(plk_state_get(h_, nullptr, nullptr, &p));
        return p;
    }

    void initZeros() { check(plk_state_zero(h_)); }
    void setBasisState(size_t index) { check(plk_state_set_basis(h_, index)); }
    void setStateVector(const std::vector<size_t> &indices, const std::vector<ComplexT> &values) {
        if (indices.size() != values.size()) pl_abort("indices and values differ in length");
        std::vector<uint64_t> idx(indices.begin(), indices.end());
        check(plk_state_set_values(h_, idx.data(), values.data(), idx.size()));
    }
    void resetStateVector() { check(plk_state_reset(h_)); }
    void HostToDevice(const ComplexT *sv, size_t length) { check(plk_state_h2d(h_, sv, length)); }
    void DeviceToHost(ComplexT *sv, size_t length) const { check(plk_state_d2h(h_, sv, length)); }
    // Queued copies (no wait; the buffer stays in use until synchronize())
    void HostToDeviceAsync(const ComplexT *sv, size_t length) { check(plk_state_h2d_async(h_, sv, length)); }
    void DeviceToHostAsync(ComplexT *sv, size_t length) const { check(plk_state_d2h_async(h_, sv, length)); }
    // The CUDA stream this state's work is queued on (nullptr: the library's)
    void setStream(void *stream) { check(plk_state_set_stream(h_, stream)); }
    void synchronize() const { check(plk_state_synchronize(h_)); }
    void DeviceToDevice(const StateVectorGB &other) { check(plk_state_copy(h_, other.h_)); }
    void updateData(const StateVectorGB &other) { DeviceToDevice(other); }

    // ---- gates --------------------------------------------------------
    void applyGate(int gate, const std::vector<size_t> &wires, bool adjoint, const std::vector<PrecisionT> &params) {
        std::vector<int64_t> w(wires.begin(), wires.end());
        std::vector<double> p(params.begin(), params.end());
        check(plk_apply_gate(h_, gate, w.data(), (int32_t)w.size(), adjoint, p.data(), (int32_t)p.size()));
    }

    void applyMatrix(const std::vector<ComplexT> &matrix, const std::vector<size_t> &wires, bool inverse = false) {
        const size_t dim = size_t(1) << wires.size();
        if (matrix.size() != dim * dim)
            pl_abort("matrix of " + std::to_string(matrix.size()) + " entries does not act on " +
                     std::to_string(wires.size()) + " wires");
        std::vector<double> m(2 * matrix.size());
        for (size_t i = 0; i < matrix.size(); i++) {
            m[2 * i] = (double)matrix[i].real();
            m[2 * i + 1] = (double)matrix[i].imag();
        }
        std::vector<int64_t> w(wires.begin(), wires.end());
        check(plk_apply_matrix(h_, m.data(), w.data(), (int32_t)w.size(), inverse));
    }

    // applyOperation :585-600: Identity is a no-op, known names run their
    // kernel, anything else is applied as the given matrix.
    void applyOperation(const std::string &name, const std::vector<size_t> &wires, bool adjoint = false,
                        const std::vector<PrecisionT> &params = {0.0}, const std::vector<ComplexT> &matrix = {}) {
        if (name == "Identity") return;
        const int g = gate_id(name);
        if (g >= 0) {
            applyGate(g, wires, adjoint, params);
            return;
        }
        if (matrix.empty()) pl_abort("Operation " + name + " has no kernel and no matrix was given");
        applyMatrix(matrix, wires, adjoint);
    }

    void applyOperation(const std::vector<std::string> &names, const std::vector<std::vector<size_t>> &wires,
                        const std::vector<bool> &adjoints, const std::vector<std::vector<PrecisionT>> &params) {
        if (names.size() != wires.size()) pl_abort("Incompatible number of ops and wires");
        if (names.size() != adjoints.size()) pl_abort("Incompatible number of ops and adjoints");
        if (names.size() != params.size()) pl_abort("Incompatible number of ops and parameters");
        std::vector<plk_op> ops;
        std::vector<std::vector<int64_t>> w(names.size());
        std::vector<std::vector<double>> p(names.size());
        for (size_t i = 0; i < names.size(); i++) {
            const int g = gate_id(names[i]);
            if (g < 0) pl_abort("Operation " + names[i] + " has no kernel");
            w[i].assign(wires[i].begin(), wires[i].end());
            p[i].assign(params[i].begin(), params[i].end());
            ops.push_back({g, (int32_t)w[i].size(), (int32_t)adjoints[i], (int32_t)p[i].size(), w[i].data(),
                           p[i].data(), nullptr});
        }
        check(plk_apply_ops(h_, ops.data(), (int32_t)ops.size()));
    }

    void applyOperation(const std::vector<std::string> &names, const std::vector<std::vector<size_t>> &wires,
                        const std::vector<bool> &adjoints) {
        std::vector<std::vector<PrecisionT>> params(names.size());
        applyOperation(names, wires, adjoints, params);
    }

    // applyGenerator :687-695; returns the scale factor
    PrecisionT applyGenerator(const std::string &name, const std::vector<size_t> &wires, bool adjoint = false,
                              const std::vector<PrecisionT> &params = {0.0}) {
        (void)params;
        const int g = gate_id(name);
        if (g < 0) pl_abort("Generator does not exist for " + name);
        std::vector<int64_t> w(wires.begin(), wires.end());
        double scale = 0.0;
        check(plk_apply_generator(h_, g, w.data(), (int32_t)w.size(), adjoint, &scale));
        return (PrecisionT)scale;
    }

  private:
    size_t num_qubits_;
    int device_;
    plk_state h_ = nullptr;
};

} // namespace Pennylane::LightningGB300
