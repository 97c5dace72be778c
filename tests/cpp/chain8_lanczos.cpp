// C++ caller of the C ABI through include/ed_hubbard.hpp, written the way the
// reference drivers are (MBL_test/src/Hubbard_test.cu): build the two H_TBq,
// the operator, run Lanczos, print E0.  Argument "--basis-only" exercises the
// host-side part without a GPU.
#include <cstdio>
#include <cstring>
#include <vector>

#include "ed_hubbard.hpp"

int main(int argc, char** argv) {
    const int N = 8, Q = 4;
    ed::H_TBq up(N, Q), dn(N, Q);
    for (int i = 0; i < N; ++i) {
        up.Make_H(i, (i + 1) % N, -1.0);
        dn.Make_H(i, (i + 1) % N, -1.0);
    }
    std::vector<uint64_t> st = up.state();
    std::printf("count %lld first %llu last %llu\n", (long long)up.count(), (unsigned long long)st.front(),
                (unsigned long long)st.back());
    if (argc > 1 && std::strcmp(argv[1], "--basis-only") == 0) return 0;
    try {
        ed::Hubbard h(up, dn, 4.0);
        ed::SpectraHubbard<double> sp(h);
        std::vector<double> x(sp.rows(), 1.0), y(sp.rows());
        sp.perform_op(x.data(), y.data());
        ed::Lanczos lanc;
        std::vector<double> evec;
        const double e0 = lanc.eigen(h, {}, evec, 100, ED_LANCZOS_FIXED, true, 0);
        std::printf("E0 %.15f steps %zu\n", e0, lanc.a.size());
    } catch (const ed::Error& e) {
        std::printf("error %d %s\n", (int)e.status, e.what());
        return 2;
    }
    return 0;
}
