// MeasuresGB.hpp — measurements over the C ABI.
//
// Mirrors MeasuresKokkos<T> (simulator/MeasuresKokkos.hpp): expectation
// values by name / matrix / CSR (:80-157), expval and var of an observable
// (:354-381), probabilities (:389-517) and sampling (:530-569).  Values are
// accumulated in FP64 on the device and returned in the state precision, as
// the reference's interface does.
#pragma once

#include <cmath>
#include <vector>

#include "ObservablesGB.hpp"

namespace Pennylane::LightningGB300 {

template <class T> class MeasuresGB {
    const StateVectorGB<T> &sv_;

  public:
    // Seed of the reference's sampler pool (MeasuresKokkos.hpp:551): every
    // call draws the same stream, as the reference's does.
    static constexpr uint64_t kDefaultSeed = 5374857ULL;

    explicit MeasuresGB(const StateVectorGB<T> &sv) : sv_(sv) {}

    // getExpectationValue(name, wires, params, matrix) :80-101
    double getExpectationValue(const std::string &name, const std::vector<size_t> &wires,
                               const std::vector<T> & /*params*/ = {0.0}, const std::vector<std::complex<T>> &matrix = {}) {
        const int g = gate_id(name);
        const bool named = g == PLK_GATE_IDENTITY || g == PLK_GATE_PAULIX || g == PLK_GATE_PAULIY ||
                           g == PLK_GATE_PAULIZ || g == PLK_GATE_HADAMARD;
        if (named) {
            std::vector<int64_t> w(wires.rbegin(), wires.rend());
            if (matrix.empty()) w.assign(wires.begin(), wires.end());
            double out = 0.0;
            check(plk_expval_named(sv_.handle(), g, w.data(), (int32_t)w.size(), &out));
            return out;
        }
        return getExpectationValue(wires, matrix);
    }

    // getExpectationValue(wires, matrix) :103-109 / MultiQubitOp :318-346
    double getExpectationValue(const std::vector<size_t> &wires, const std::vector<std::complex<T>> &matrix) {
        const size_t dim = size_t(1) << wires.size();
        if (matrix.size() != dim * dim) pl_abort("observable matrix size does not match the wire count");
        std::vector<double> m(2 * matrix.size());
        for (size_t i = 0; i < matrix.size(); i++) {
            m[2 * i] = matrix[i].real();
            m[2 * i + 1] = matrix[i].imag();
        }
        std::vector<int64_t> w(wires.begin(), wires.end());
        double out = 0.0;
        check(plk_expval_matrix(sv_.handle(), m.data(), w.data(), (int32_t)w.size(), &out));
        return out;
    }

    // getExpectationValue(data, indices, index_ptr) :111-135
    double getExpectationValue(const std::vector<std::complex<T>> &data, const std::vector<size_t> &indices,
                               const std::vector<size_t> &index_ptr) {
        std::vector<double> d(2 * data.size());
        for (size_t i = 0; i < data.size(); i++) {
            d[2 * i] = data[i].real();
            d[2 * i + 1] = data[i].imag();
        }
        std::vector<int64_t> ind(indices.begin(), indices.end()), ptr(index_ptr.begin(), index_ptr.end());
        if (ptr.empty()) pl_abort("empty index_ptr");
        double out = 0.0;
        check(plk_expval_sparse(sv_.handle(), d.data(), ind.data(), ptr.data(), (int64_t)ptr.size() - 1,
                                (int64_t)ind.size(), &out));
        return out;
    }

    double pauliSum(const std::vector<PauliWord> &words) {
        std::vector<double> c;
        std::vector<int64_t> off{0}, w;
        std::string letters;
        for (const auto &pw : words) {
            c.push_back(pw.coeff);
            for (size_t j = 0; j < pw.wires.size(); j++) {
                w.push_back((int64_t)pw.wires[j]);
                letters.push_back(pw.letters[j]);
            }
            off.push_back((int64_t)w.size());
        }
        double out = 0.0;
        check(plk_expval_pauli_sum(sv_.handle(), (int32_t)c.size(), c.data(), off.data(), w.data(), letters.data(),
                                   &out));
        return out;
    }

    // expval(ob) :354-360: Re<psi|O psi>; Pauli sums skip the state copy.
    double expval(const ObservableGB<T> &ob) {
        if (auto words = ob.pauliWords()) return pauliSum(*words);
        StateVectorGB<T> ob_sv(sv_);
        ob.applyInPlace(ob_sv);
        double re = 0.0;
        check(plk_inner_product(sv_.handle(), ob_sv.handle(), &re, nullptr));
        return re;
    }

    // var(ob) :368-381
    double var(const ObservableGB<T> &ob) {
        StateVectorGB<T> ob_sv(sv_);
        ob.applyInPlace(ob_sv);
        double ms = 0.0, mean = 0.0;
        check(plk_inner_product(ob_sv.handle(), ob_sv.handle(), &ms, nullptr));
        check(plk_inner_product(sv_.handle(), ob_sv.handle(), &mean, nullptr));
        return ms - mean * mean;
    }

    std::vector<double> probs(const std::vector<size_t> &wires = {}) {
        std::vector<int64_t> w(wires.begin(), wires.end());
        std::vector<double> out(size_t(1) << (w.empty() ? sv_.getNumQubits() : w.size()));
        check(plk_probs(sv_.handle(), w.data(), (int32_t)w.size(), out.data()));
        return out;
    }

    std::vector<int64_t> generate_samples(size_t num_samples, uint64_t seed = kDefaultSeed) {
        std::vector<int64_t> out(num_samples * sv_.getNumQubits());
        check(plk_generate_samples(sv_.handle(), num_samples, seed, out.data()));
        return out;
    }

    std::vector<int64_t> samples_from_uniforms(const std::vector<double> &u) {
        std::vector<int64_t> out(u.size() * sv_.getNumQubits());
        check(plk_sample_from_uniforms(sv_.handle(), u.data(), u.size(), out.data()));
        return out;
    }
};

} // namespace Pennylane::LightningGB300
