// Driver for the GPU test of the C++ host layer (MeasuresGB::expval / var,
// the observable classes) on a caller-given state.
//
// Usage: host_measures <64|128> <state.bin> <herm.bin>
//   state.bin: 2^n complex128 amplitudes; herm.bin: a 4 x 4 complex128
//   matrix (row-major) for a two-wire Hermitian observable.
// Prints one line per observable: "<label> <expval> <var>" with 17 digits.
#include <complex>
#include <cstdio>
#include <fstream>
#include <iterator>
#include <memory>
#include <vector>

#include "host/MeasuresGB.hpp"

using namespace Pennylane::LightningGB300;

static std::vector<std::complex<double>> read_c128(const char *path) {
    std::ifstream f(path, std::ios::binary);
    std::vector<char> raw((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<std::complex<double>> out(raw.size() / sizeof(std::complex<double>));
    std::copy(raw.begin(), raw.begin() + out.size() * sizeof(std::complex<double>), (char *)out.data());
    return out;
}

template <class T> static int run(const char *state_path, const char *herm_path) {
    using C = std::complex<T>;
    const auto psi64 = read_c128(state_path);
    const auto herm64 = read_c128(herm_path);
    std::vector<C> psi(psi64.begin(), psi64.end());
    std::vector<C> herm(herm64.begin(), herm64.end());
    StateVectorGB<T> sv(psi.data(), psi.size());
    MeasuresGB<T> m(sv);
    using Obs = std::shared_ptr<ObservableGB<T>>;
    Obs x1 = std::make_shared<NamedObsGB<T>>("PauliX", std::vector<size_t>{1});
    Obs z0 = std::make_shared<NamedObsGB<T>>("PauliZ", std::vector<size_t>{0});
    Obs y2 = std::make_shared<NamedObsGB<T>>("PauliY", std::vector<size_t>{2});
    Obs h4 = std::make_shared<NamedObsGB<T>>("Hadamard", std::vector<size_t>{4});
    Obs zy = std::make_shared<TensorProdObsGB<T>>(std::vector<Obs>{z0, y2});
    Obs he = std::make_shared<HermitianObsGB<T>>(herm, std::vector<size_t>{3, 1});
    Obs ham = std::make_shared<HamiltonianGB<T>>(std::vector<T>{0.7, -1.3, 0.4}, std::vector<Obs>{x1, zy, he});
    const std::pair<const char *, Obs> list[] = {{"x1", x1}, {"h4", h4}, {"zy", zy}, {"herm", he}, {"ham", ham}};
    for (const auto &[label, ob] : list) std::printf("%s %.17g %.17g\n", label, m.expval(*ob), m.var(*ob));
    return 0;
}

int main(int argc, char **argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: host_measures <64|128> <state.bin> <herm.bin>\n");
        return 2;
    }
    try {
        return std::string(argv[1]) == "64" ? run<float>(argv[2], argv[3]) : run<double>(argv[2], argv[3]);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
