// ObservablesGB.hpp — observable classes over the C ABI.
//
// Mirrors simulator/ObservablesKokkos.hpp: NamedObs (:77-119),
// HermitianObs (:124-180), TensorProdObs (:185-290), Hamiltonian
// (:296-402), SparseHamiltonian (:409-517), with the same applyInPlace
// semantics.  Observables built only from Pauli letters additionally expose
// their Pauli-word form, which lets expectation values and H|psi> run as
// single-pass Pauli-sum kernels instead of the copy/apply/axpy loop.
#pragma once

#include <algorithm>
#include <functional>
#include <iomanip>
#include <memory>
#include <optional>
#include <set>
#include <sstream>
#include <string>
#include <typeinfo>
#include <vector>

#include "StateVectorGB.hpp"

namespace Pennylane::LightningGB300 {

// A weighted product of Pauli letters on distinct wires.
struct PauliWord {
    double coeff = 1.0;
    std::vector<size_t> wires;
    std::string letters;
};

template <class T> inline std::string vec_str(const std::vector<T> &v) {
    std::ostringstream ss;
    ss << "[";
    for (size_t i = 0; i < v.size(); i++) ss << v[i] << (i + 1 < v.size() ? ", " : "");
    ss << "]";
    return ss.str();
}

template <class T> class ObservableGB : public std::enable_shared_from_this<ObservableGB<T>> {
  public:
    virtual ~ObservableGB() = default;
    virtual void applyInPlace(StateVectorGB<T> &sv) const = 0;
    [[nodiscard]] virtual std::string getObsName() const = 0;
    [[nodiscard]] virtual std::vector<size_t> getWires() const = 0;
    // Pauli-sum form, if the observable is one (nullopt otherwise)
    [[nodiscard]] virtual std::optional<std::vector<PauliWord>> pauliWords() const { return std::nullopt; }
    [[nodiscard]] bool operator==(const ObservableGB<T> &other) const {
        return typeid(*this) == typeid(other) && isEqual(other);
    }
    [[nodiscard]] bool operator!=(const ObservableGB<T> &other) const { return !(*this == other); }

  private:
    [[nodiscard]] virtual bool isEqual(const ObservableGB<T> &other) const = 0;
};

template <class T> class NamedObsGB final : public ObservableGB<T> {
    std::string name_;
    std::vector<size_t> wires_;
    std::vector<T> params_;

    [[nodiscard]] bool isEqual(const ObservableGB<T> &o) const override {
        const auto &c = static_cast<const NamedObsGB<T> &>(o);
        return name_ == c.name_ && wires_ == c.wires_ && params_ == c.params_;
    }

  public:
    NamedObsGB(std::string name, std::vector<size_t> wires, std::vector<T> params = {})
        : name_(std::move(name)), wires_(std::move(wires)), params_(std::move(params)) {}
    [[nodiscard]] std::string getObsName() const override { return name_ + vec_str(wires_); }
    [[nodiscard]] std::vector<size_t> getWires() const override { return wires_; }
    [[nodiscard]] const std::string &name() const { return name_; }
    void applyInPlace(StateVectorGB<T> &sv) const override { sv.applyOperation(name_, wires_, false, params_); }
    [[nodiscard]] std::optional<std::vector<PauliWord>> pauliWords() const override {
        PauliWord w;
        if (name_ == "Identity") return std::vector<PauliWord>{w};
        if (wires_.size() != 1) return std::nullopt;
        char l = 0;
        if (name_ == "PauliX") l = 'X';
        else if (name_ == "PauliY") l = 'Y';
        else if (name_ == "PauliZ") l = 'Z';
        else return std::nullopt;
        w.wires = wires_;
        w.letters = std::string(1, l);
        return std::vector<PauliWord>{w};
    }
};

template <class T> class HermitianObsGB final : public ObservableGB<T> {
  public:
    using MatrixT = std::vector<std::complex<T>>;

  private:
    MatrixT matrix_;
    std::vector<size_t> wires_;

    [[nodiscard]] bool isEqual(const ObservableGB<T> &o) const override {
        const auto &c = static_cast<const HermitianObsGB<T> &>(o);
        return matrix_ == c.matrix_ && wires_ == c.wires_;
    }

  public:
    HermitianObsGB(MatrixT matrix, std::vector<size_t> wires) : matrix_(std::move(matrix)), wires_(std::move(wires)) {}
    [[nodiscard]] const MatrixT &getMatrix() const { return matrix_; }
    [[nodiscard]] std::vector<size_t> getWires() const override { return wires_; }
    [[nodiscard]] std::string getObsName() const override {
        // MatrixHasher (util/UtilKokkos.hpp:61-72): combine the hashes of the entries
        size_t h = 0;
        for (const auto &z : matrix_) {
            h ^= std::hash<T>{}(z.real()) + 0x9e3779b9 + (h << 6) + (h >> 2);
            h ^= std::hash<T>{}(z.imag()) + 0x9e3779b9 + (h << 6) + (h >> 2);
        }
        std::ostringstream ss;
        ss << "Hermitian" << h;
        return ss.str();
    }
    void applyInPlace(StateVectorGB<T> &sv) const override { sv.applyMatrix(matrix_, wires_, false); }
};

template <class T> class TensorProdObsGB final : public ObservableGB<T> {
    std::vector<std::shared_ptr<ObservableGB<T>>> obs_;
    std::vector<size_t> all_wires_;

    [[nodiscard]] bool isEqual(const ObservableGB<T> &o) const override {
        const auto &c = static_cast<const TensorProdObsGB<T> &>(o);
        if (obs_.size() != c.obs_.size()) return false;
        for (size_t i = 0; i < obs_.size(); i++)
            if (*obs_[i] != *c.obs_[i]) return false;
        return true;
    }

  public:
    explicit TensorProdObsGB(std::vector<std::shared_ptr<ObservableGB<T>>> obs) : obs_(std::move(obs)) {
        std::set<size_t> wires;
        for (const auto &ob : obs_)
            for (size_t w : ob->getWires()) {
                if (wires.count(w)) pl_abort("All wires in observables must be disjoint.");
                wires.insert(w);
            }
        all_wires_.assign(wires.begin(), wires.end());
    }
    [[nodiscard]] size_t getSize() const { return obs_.size(); }
    [[nodiscard]] std::vector<size_t> getWires() const override { return all_wires_; }
    void applyInPlace(StateVectorGB<T> &sv) const override {
        for (const auto &ob : obs_) ob->applyInPlace(sv);
    }
    [[nodiscard]] std::string getObsName() const override {
        std::ostringstream ss;
        for (size_t i = 0; i < obs_.size(); i++) ss << obs_[i]->getObsName() << (i + 1 < obs_.size() ? " @ " : "");
        return ss.str();
    }
    [[nodiscard]] std::optional<std::vector<PauliWord>> pauliWords() const override {
        PauliWord w;
        for (const auto &ob : obs_) {
            auto sub = ob->pauliWords();
            if (!sub || sub->size() != 1) return std::nullopt;
            const PauliWord &s = (*sub)[0];
            w.coeff *= s.coeff;
            w.wires.insert(w.wires.end(), s.wires.begin(), s.wires.end());
            w.letters += s.letters;
        }
        return std::vector<PauliWord>{w};
    }
};

template <class T> class HamiltonianGB final : public ObservableGB<T> {
    std::vector<T> coeffs_;
    std::vector<std::shared_ptr<ObservableGB<T>>> obs_;

    [[nodiscard]] bool isEqual(const ObservableGB<T> &o) const override {
        const auto &c = static_cast<const HamiltonianGB<T> &>(o);
        if (coeffs_ != c.coeffs_ || obs_.size() != c.obs_.size()) return false;
        for (size_t i = 0; i < obs_.size(); i++)
            if (*obs_[i] != *c.obs_[i]) return false;
        return true;
    }

  public:
    HamiltonianGB(std::vector<T> coeffs, std::vector<std::shared_ptr<ObservableGB<T>>> obs)
        : coeffs_(std::move(coeffs)), obs_(std::move(obs)) {
        if (coeffs_.size() != obs_.size()) pl_abort("Hamiltonian coefficients and terms differ in number");
    }
    // HamiltonianKokkos::applyInPlace :360-373: sv <- sum_j c_j O_j sv.  Pauli
    // sums run as one Pauli-sum kernel (no per-term state copies).
    void applyInPlace(StateVectorGB<T> &sv) const override {
        StateVectorGB<T> buffer(sv.getNumQubits(), InitializationSettings{0, sv.device()});
        if (auto words = pauliWords()) {
            applyPauliWords(buffer, sv, *words);
        } else {
            buffer.initZeros();
            for (size_t t = 0; t < coeffs_.size(); t++) {
                StateVectorGB<T> tmp(sv);
                obs_[t]->applyInPlace(tmp);
                check(plk_state_axpy(buffer.handle(), (double)coeffs_[t], 0.0, tmp.handle()));
            }
        }
        sv.updateData(buffer);
    }
    static void applyPauliWords(StateVectorGB<T> &out, const StateVectorGB<T> &in, const std::vector<PauliWord> &words) {
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
        check(plk_apply_pauli_sum(out.handle(), in.handle(), (int32_t)c.size(), c.data(), off.data(), w.data(),
                                  letters.data()));
    }
    [[nodiscard]] std::vector<size_t> getWires() const override {
        std::set<size_t> wires;
        for (const auto &ob : obs_)
            for (size_t x : ob->getWires()) wires.insert(x);
        return {wires.begin(), wires.end()};
    }
    [[nodiscard]] std::string getObsName() const override {
        std::ostringstream ss;
        ss << "Hamiltonian: { 'coeffs' : " << vec_str(coeffs_) << ", 'observables' : [";
        for (size_t t = 0; t < obs_.size(); t++) ss << obs_[t]->getObsName() << (t + 1 < obs_.size() ? ", " : "");
        ss << "]}";
        return ss.str();
    }
    [[nodiscard]] std::optional<std::vector<PauliWord>> pauliWords() const override {
        std::vector<PauliWord> out;
        for (size_t t = 0; t < obs_.size(); t++) {
            auto sub = obs_[t]->pauliWords();
            if (!sub) return std::nullopt;
            for (auto w : *sub) {
                w.coeff *= (double)coeffs_[t];
                out.push_back(std::move(w));
            }
        }
        return out;
    }
};

template <class T> class SparseHamiltonianGB final : public ObservableGB<T> {
    std::vector<std::complex<T>> data_;
    std::vector<size_t> indices_, indptr_, wires_;

    [[nodiscard]] bool isEqual(const ObservableGB<T> &o) const override {
        const auto &c = static_cast<const SparseHamiltonianGB<T> &>(o);
        return data_ == c.data_ && indices_ == c.indices_ && indptr_ == c.indptr_;
    }

  public:
    SparseHamiltonianGB(std::vector<std::complex<T>> data, std::vector<size_t> indices, std::vector<size_t> indptr,
                        std::vector<size_t> wires)
        : data_(std::move(data)), indices_(std::move(indices)), indptr_(std::move(indptr)), wires_(std::move(wires)) {
        if (data_.size() != indices_.size()) pl_abort("sparse data and indices differ in length");
    }
    // SparseHamiltonianKokkos::applyInPlace :484-494
    void applyInPlace(StateVectorGB<T> &sv) const override {
        if (wires_.size() != sv.getNumQubits()) pl_abort("SparseH wire count does not match state-vector size");
        StateVectorGB<T> out(sv.getNumQubits(), InitializationSettings{0, sv.device()});
        std::vector<double> d(2 * data_.size());
        for (size_t i = 0; i < data_.size(); i++) {
            d[2 * i] = data_[i].real();
            d[2 * i + 1] = data_[i].imag();
        }
        std::vector<int64_t> ind(indices_.begin(), indices_.end()), ptr(indptr_.begin(), indptr_.end());
        check(plk_spmv(out.handle(), sv.handle(), d.data(), ind.data(), ptr.data(), (int64_t)ptr.size() - 1,
                       (int64_t)ind.size()));
        sv.updateData(out);
    }
    [[nodiscard]] std::string getObsName() const override {
        std::ostringstream ss;
        ss << "SparseHamiltonian: {\n'data' : ";
        for (const auto &d : data_) ss << d;
        ss << ",\n'indices' : ";
        for (const auto &i : indices_) ss << i;
        ss << ",\n'indptr' : ";
        for (const auto &o : indptr_) ss << o;
        ss << "\n}";
        return ss.str();
    }
    [[nodiscard]] std::vector<size_t> getWires() const override { return wires_; }
    [[nodiscard]] const std::vector<std::complex<T>> &data() const { return data_; }
    [[nodiscard]] const std::vector<size_t> &indices() const { return indices_; }
    [[nodiscard]] const std::vector<size_t> &indptr() const { return indptr_; }
};

} // namespace Pennylane::LightningGB300
