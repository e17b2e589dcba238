// AdjointGB.hpp — adjoint-method Jacobian over the C ABI.
//
// Mirrors OpsData<T> and AdjointJacobianKokkos<T>
// (algorithms/AdjointDiffKokkos.hpp:17-478).  The host side builds
// H_lambda_i = O_i |lambda> for each observable (Pauli sums in one kernel,
// other observables through applyInPlace) and hands the serialised tape to
// plk_adjoint_jacobian, which runs the fused backward sweep on the GPU.
// Differences from the reference, both fixes of documented quirks:
//  - ops without a kernel are applied through the matrix stored in OpsData
//    (the reference drops ops_matrices, AdjointDiffKokkos.hpp:223-226);
//  - StatePrep / BasisState entries are skipped as in :447-450.
#pragma once

#include <numeric>
#include <string>
#include <vector>

#include "MeasuresGB.hpp"

namespace Pennylane::LightningGB300 {

template <class T> class OpsData {
    std::vector<std::string> names_;
    std::vector<std::vector<T>> params_;
    std::vector<std::vector<size_t>> wires_;
    std::vector<bool> inverses_;
    std::vector<std::vector<std::complex<T>>> matrices_;
    size_t num_par_ops_ = 0;

  public:
    OpsData(std::vector<std::string> names, std::vector<std::vector<T>> params, std::vector<std::vector<size_t>> wires,
            std::vector<bool> inverses, std::vector<std::vector<std::complex<T>>> matrices = {})
        : names_(std::move(names)), params_(std::move(params)), wires_(std::move(wires)), inverses_(std::move(inverses)),
          matrices_(std::move(matrices)) {
        if (matrices_.empty()) matrices_.resize(names_.size());
        if (params_.size() != names_.size() || wires_.size() != names_.size() || inverses_.size() != names_.size() ||
            matrices_.size() != names_.size())
            pl_abort("OpsData: names, params, wires, inverses and matrices differ in length");
        for (const auto &p : params_)
            if (!p.empty()) num_par_ops_++;
    }
    [[nodiscard]] size_t getSize() const { return names_.size(); }
    [[nodiscard]] const std::vector<std::string> &getOpsName() const { return names_; }
    [[nodiscard]] const std::vector<std::vector<T>> &getOpsParams() const { return params_; }
    [[nodiscard]] const std::vector<std::vector<size_t>> &getOpsWires() const { return wires_; }
    [[nodiscard]] const std::vector<bool> &getOpsInverses() const { return inverses_; }
    [[nodiscard]] const std::vector<std::vector<std::complex<T>>> &getOpsMatrices() const { return matrices_; }
    [[nodiscard]] bool hasParams(size_t i) const { return !params_[i].empty(); }
    [[nodiscard]] size_t getNumParOps() const { return num_par_ops_; }
    [[nodiscard]] size_t getNumNonParOps() const { return names_.size() - num_par_ops_; }
    [[nodiscard]] size_t getTotalNumParams() const {
        return std::accumulate(params_.begin(), params_.end(), size_t{0},
                               [](size_t a, const std::vector<T> &p) { return a + p.size(); });
    }
};

template <class T> class AdjointJacobianGB {
  public:
    OpsData<T> createOpsData(const std::vector<std::string> &names, const std::vector<std::vector<T>> &params,
                             const std::vector<std::vector<size_t>> &wires, const std::vector<bool> &inverses,
                             const std::vector<std::vector<std::complex<T>>> &matrices = {}) {
        return OpsData<T>(names, params, wires, inverses, matrices);
    }

    // jac[obs][trainable]; apply_operations = true first runs the tape on a
    // copy of ref_data (AdjointDiffKokkos.hpp:429-431).
    void adjointJacobian(const StateVectorGB<T> &ref_data, std::vector<std::vector<T>> &jac,
                         const std::vector<std::shared_ptr<ObservableGB<T>>> &obs, const OpsData<T> &ops,
                         const std::vector<size_t> &trainable, bool apply_operations = false) {
        std::vector<double> flat;
        adjointJacobianFlat(ref_data, flat, obs, ops, trainable, apply_operations);
        jac.assign(obs.size(), std::vector<T>(trainable.size(), 0));
        for (size_t o = 0; o < obs.size(); o++)
            for (size_t t = 0; t < trainable.size(); t++) jac[o][t] = (T)flat[o * trainable.size() + t];
    }

    // The same, into a row-major FP64 buffer [num_obs][num_trainable].
    void adjointJacobianFlat(const StateVectorGB<T> &ref_data, std::vector<double> &jac,
                             const std::vector<std::shared_ptr<ObservableGB<T>>> &obs, const OpsData<T> &ops,
                             const std::vector<size_t> &trainable, bool apply_operations = false) {
        if (trainable.empty()) pl_abort("No trainable parameters provided.");
        if (obs.empty()) {
            jac.clear();
            return;
        }
        // serialise the tape
        const size_t n = ops.getSize();
        std::vector<plk_op> tape;
        std::vector<std::vector<int64_t>> w(n);
        std::vector<std::vector<double>> p(n), m(n);
        for (size_t i = 0; i < n; i++) {
            const std::string &name = ops.getOpsName()[i];
            if (name == "StatePrep" || name == "BasisState" || name == "QubitStateVector") continue;
            int g = gate_id(name);
            w[i].assign(ops.getOpsWires()[i].begin(), ops.getOpsWires()[i].end());
            p[i].assign(ops.getOpsParams()[i].begin(), ops.getOpsParams()[i].end());
            const double *mat = nullptr;
            if (g < 0) {
                const auto &mm = ops.getOpsMatrices()[i];
                if (mm.empty()) pl_abort("Operation " + name + " has neither a kernel nor a matrix");
                m[i].resize(2 * mm.size());
                for (size_t k = 0; k < mm.size(); k++) {
                    m[i][2 * k] = mm[k].real();
                    m[i][2 * k + 1] = mm[k].imag();
                }
                g = PLK_GATE_MATRIX;
                mat = m[i].data();
            }
            tape.push_back({g, (int32_t)w[i].size(), (int32_t)ops.getOpsInverses()[i], (int32_t)p[i].size(),
                            w[i].data(), p[i].data(), mat});
        }
        StateVectorGB<T> lambda(ref_data);
        if (apply_operations) check(plk_apply_ops(lambda.handle(), tape.data(), (int32_t)tape.size()));
        // H_lambda states
        std::vector<std::unique_ptr<StateVectorGB<T>>> hl;
        std::vector<plk_state> hh;
        for (const auto &ob : obs) {
            if (auto words = ob->pauliWords()) {
                hl.emplace_back(new StateVectorGB<T>(lambda.getNumQubits(), InitializationSettings{0, lambda.device()}));
                HamiltonianGB<T>::applyPauliWords(*hl.back(), lambda, *words);
            } else {
                hl.emplace_back(new StateVectorGB<T>(lambda));
                ob->applyInPlace(*hl.back());
            }
            hh.push_back(hl.back()->handle());
        }
        std::vector<int64_t> tp(trainable.begin(), trainable.end());
        jac.assign(obs.size() * trainable.size(), 0.0);
        check(plk_adjoint_jacobian(lambda.handle(), hh.data(), (int32_t)hh.size(), tape.data(), (int32_t)tape.size(),
                                   tp.data(), (int32_t)tp.size(), jac.data()));
    }
};

} // namespace Pennylane::LightningGB300
