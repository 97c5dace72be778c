// C++ caller of the C ABI through include/ed_hubbard.hpp, written the way the
// reference drivers are (MBL_test/src/Hubbard_test.cu): build the two H_TBq,
// the operator, run Lanczos, print E0 and the entanglement entropy; then the
// three lowest eigenpairs (TotalSpinExcited_*) and one Krylov time step
// (Time_evol_test.cu).
// Argument "--basis-only" exercises the host-side part without a GPU.
#include <cstdio>
#include <algorithm>
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
        // Hubbard_EE_test.cu: entanglement of sites 0..3, one state and a batch of two
        const auto ee = ed::entanglement_entropy(h, evec, 0x0Fu);
        std::vector<double> two(evec);
        two.insert(two.end(), evec.begin(), evec.end());
        std::vector<double> bvn, bref;
        ed::entanglement_entropy_batch(h, 2, two, 0x0Fu, bvn, bref);
        std::printf("EE %.15f %.15f %d %d\n", ee.first, ee.second, (int)(bvn[0] == ee.first && bvn[1] == ee.first),
                    h.matvec_kind());
        // the drivers' loop over samples and sectors as one batched launch: the
        // 4+4 operator and a 5+3 one, each run equal to its own
        ed::H_TBq up5(N, 5), dn3(N, 3);
        for (int i = 0; i < N; ++i) {
            up5.Make_H(i, (i + 1) % N, -1.0);
            dn3.Make_H(i, (i + 1) % N, -1.0);
        }
        ed::Hubbard h53(up5, dn3, 4.0);
        std::vector<double> bev;
        const std::vector<double> be0 = ed::lanczos_batch({&h, &h53}, 60, {}, bev, 11);
        ed::Lanczos l0, l1;
        std::vector<double> v0, v1;
        l0.eigen(h, {}, v0, 60, ED_LANCZOS_FIXED, false, 11);
        l1.eigen(h53, {}, v1, 60, ED_LANCZOS_FIXED, false, 12);
        const bool same = be0[0] == l0.result.e0 && be0[1] == l1.result.e0 &&
                          std::equal(v0.begin(), v0.end(), bev.begin()) &&
                          std::equal(v1.begin(), v1.end(), bev.begin() + v0.size());
        std::printf("BATCH %.15f %.15f %d\n", be0[0], be0[1], (int)same);
        // TotalSpinExcited_*: the lowest pairs through the Spectra-shaped solver
        ed::SymEigsSolver eigs(h, 3, 4 * (3 + 1));
        eigs.init();
        const int nconv = eigs.compute(1000, 1e-10);
        std::printf("EIGS %d %.15f %.15f %.15f\n", nconv, eigs.eigenvalues()[0], eigs.eigenvalues()[1],
                    eigs.eigenvalues()[2]);
        // Time_evol_test.cu: exp(-i H t) on a product state, host vectors through the C ABI
        std::vector<double> phi0(2 * sp.rows(), 0.0), phi(2 * sp.rows());
        phi0[0] = 1.0;
        ed_krylov_cfg kc{200, 0, 1e-12, 0, 0};
        ed_krylov_result kr{};
        const double t = 0.5;
        if (ed_krylov_evolve(h.handle(), &kc, phi0.data(), ED_MEM_HOST, 1, &t, phi.data(), ED_MEM_HOST, &kr, nullptr) !=
            ED_OK)
            return 3;
        double nrm = 0.0;
        for (double v : phi) nrm += v * v;
        std::printf("KRYLOV steps %d norm2 %.15f\n", kr.steps, nrm);
    } catch (const ed::Error& e) {
        std::printf("error %d %s\n", (int)e.status, e.what());
        return 2;
    }
    return 0;
}
