// ed_hubbard.hpp — header-only C++ surface over the C ABI in ed_hubbard.h,
// shaped like the reference's own classes so its drivers switch by changing
// types, not call sites:
//   ed::H_TBq                Make_H / Make_J / Make_N, state  (fermi_operator.h:42-242)
//   ed::Hubbard              Hubbard(HqUP, HqDN, U[, dilution]), Hubbard_mv(x, y) on
//                            device pointers                  (HubMatrix_GPU.cuh:30-182)
//   ed::SpectraHubbard<T>    Scalar, rows(), cols(), perform_op(x, y) on host
//                            pointers — the Spectra operator concept
//                                                             (HubMatrix_TotalSpin.cuh:181-322)
//   ed::Lanczos              random_vector / eigen            (HubMatrix_GPU.cuh:477-613)
//   ed::Krylov               Make_tridiagonal_eigen / Krylov_time_evol on device
//                            complex vectors                  (HubMatrix_GPU.cuh:619-728)
//   ed::SymEigsSolver        init / compute / eigenvalues / eigenvectors / info,
//                            the nev lowest pairs on the device (Spectra::SymEigsSolver
//                            as TotalSpinExcited_Lieb_randomHop.cu:133-143 uses it)
// Errors surface as ed::Error (std::runtime_error) carrying the ed_status.
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ed_hubbard.h"

namespace ed {

struct Error : std::runtime_error {
    ed_status status;
    Error(ed_status s, const char* where)
        : std::runtime_error(std::string(where) + ": " + ed_status_string(s)), status(s) {}
};

inline void check(ed_status s, const char* where) {
    if (s != ED_OK) throw Error(s, where);
}

class H_TBq {
public:
    int N, Q;
    H_TBq(int n, int q) : N(n), Q(q) {}
    void Make_H(int i, int j, double t) { terms_.push_back({ED_TERM_HOP, i, j, 0, t, 0.0}); }
    void Make_J(int i, int j, double t) { terms_.push_back({ED_TERM_CURRENT, i, j, 0, t, 0.0}); }
    void Make_N(int i, double v) { terms_.push_back({ED_TERM_DENSITY, i, 0, 0, v, 0.0}); }
    void Make_Peierls(int i, int j, double t, double phase) {
        terms_.push_back({ED_TERM_PEIERLS, i, j, 0, t, phase});
    }
    void clear() { terms_.clear(); }
    int64_t count() const { return ed_binom(N, Q); }
    std::vector<uint64_t> state() const {
        std::vector<int64_t> r(count());
        for (int64_t k = 0; k < (int64_t)r.size(); ++k) r[k] = k;
        std::vector<uint64_t> w(r.size());
        check(ed_basis_unrank(N, Q, r.data(), (int64_t)r.size(), w.data()), "ed_basis_unrank");
        return w;
    }
    const std::vector<ed_term>& terms() const { return terms_; }

private:
    std::vector<ed_term> terms_;
};

class Hubbard {
public:
    Hubbard(const H_TBq& up, const H_TBq& dn, double U = 0.0, uint64_t dilution = 0, int device = 0,
            bool complex_op = false) {
        ed_model_desc d{};
        d.n_sites = up.N;
        d.n_up = up.Q;
        d.n_dn = dn.Q;
        d.flags = complex_op ? ED_OP_COMPLEX : ED_OP_REAL;
        d.up_terms = up.terms().data();
        d.n_up_terms = (int32_t)up.terms().size();
        d.dn_terms = dn.terms().data();
        d.n_dn_terms = (int32_t)dn.terms().size();
        d.U = U;
        d.interaction_mask = dilution;
        check(ed_op_create(&op_, &d, device), "ed_op_create");
    }
    Hubbard(const Hubbard&) = delete;
    Hubbard& operator=(const Hubbard&) = delete;
    ~Hubbard() { ed_op_destroy(op_); }
    // y = H x on device vectors, asynchronous on `stream` (cudaStream_t)
    void Hubbard_mv(const double* x, double* y, void* stream = nullptr) {
        check(ed_op_perform(op_, x, y, ED_MEM_DEVICE, stream), "Hubbard_mv");
    }
    int64_t rows() const { return ed_op_rows(op_); }
    int64_t cols() const { return ed_op_cols(op_); }
    int64_t dimUP() const { return ed_op_dim_up(op_); }
    int64_t dimDN() const { return ed_op_dim_dn(op_); }
    // ED_MV_ROWS, ED_MV_TWO_PASS or ED_MV_GENERIC: the matvec of its Lanczos steps
    int matvec_kind() const { return ed_op_matvec_kind(op_); }
    ed_op* handle() const { return op_; }

private:
    ed_op* op_ = nullptr;
};

// The Spectra operator concept on host pointers (synchronous, y overwritten):
// usable as Spectra::SymEigsSolver<ed::SpectraHubbard<double>>.
template <typename FloatType = double>
class SpectraHubbard {
    static_assert(sizeof(FloatType) == sizeof(double), "FP64 operator");

public:
    using Scalar = FloatType;
    explicit SpectraHubbard(Hubbard& h) : h_(h) {}
    int64_t rows() const { return h_.rows(); }
    int64_t cols() const { return h_.cols(); }
    void perform_op(const Scalar* x, Scalar* y) const {
        check(ed_op_perform(h_.handle(), reinterpret_cast<const double*>(x), reinterpret_cast<double*>(y),
                            ED_MEM_HOST, nullptr),
              "perform_op");
    }

private:
    Hubbard& h_;
};

class Lanczos {
public:
    std::vector<double> a, b;  // T: alpha, beta (b[0] = |f|)
    ed_lanczos_result result{};
    // uniform(-1,1) from Philox4x64-10(seed), normalised
    static std::vector<double> random_vector(int64_t n, uint64_t seed = 0) {
        std::vector<double> f(n);
        check(ed_random_vector(n, seed, f.data()), "ed_random_vector");
        double s = 0.0;
        for (double v : f) s += v * v;
        s = 1.0 / std::sqrt(s);
        for (double& v : f) v *= s;
        return f;
    }
    // The reference's eigen(): stop test every 10 steps, up to max_steps;
    // f (host, may be empty for the seeded random start); evec (host) out.
    double eigen(Hubbard& h, const std::vector<double>& f, std::vector<double>& evec, int max_steps = 1000,
                 int mode = ED_LANCZOS_REFERENCE, bool reorth = false, uint64_t seed = 0) {
        ed_lanczos_cfg cfg{};
        cfg.max_steps = max_steps;
        cfg.mode = mode;
        cfg.reorth = reorth ? 1 : 0;
        cfg.ritz = ED_RITZ_STORED;
        cfg.start = f.empty() ? ED_START_RANDOM : ED_START_USER;
        cfg.seed = seed;
        evec.resize(h.rows());
        a.assign(max_steps, 0.0);
        b.assign(max_steps + 1, 0.0);
        check(ed_lanczos_run(h.handle(), &cfg, f.empty() ? nullptr : f.data(), ED_MEM_HOST, evec.data(), ED_MEM_HOST,
                             a.data(), b.data(), &result, nullptr),
              "ed_lanczos_run");
        a.resize(result.steps);
        b.resize(result.steps + 1);
        return result.e0;
    }
};

// Entanglement entropy of a host state for the sites in a_mask
// (EEmatHubAB_GPU::Make_Write + cusolverDsvd + the entropy sum of
// Hubbard_EE_test.cu:78-83): {S_vN = -sum s^2 ln s^2, S_ref = -sum s ln s}.
inline std::pair<double, double> entanglement_entropy(Hubbard& h, const std::vector<double>& psi, uint64_t a_mask) {
    double svn = 0.0, sref = 0.0;
    check(ed_entanglement_entropy(h.handle(), psi.data(), ED_MEM_HOST, a_mask, &svn, &sref, nullptr),
          "ed_entanglement_entropy");
    return {svn, sref};
}

// The same for n states of h's sector stored one after another in psis
// (host, n x rows), in one batched call; each value equals its own call's.
inline void entanglement_entropy_batch(Hubbard& h, int n, const std::vector<double>& psis, uint64_t a_mask,
                                       std::vector<double>& s_vn, std::vector<double>& s_ref) {
    s_vn.assign(n, 0.0);
    s_ref.assign(n, 0.0);
    check(ed_entanglement_entropy_batch(h.handle(), n, psis.data(), ED_MEM_HOST, a_mask, s_vn.data(), s_ref.data(),
                                        nullptr),
          "ed_entanglement_entropy_batch");
}

// Fixed-step Lanczos runs of up to 16 operators (any sectors, real or complex)
// in one persistent launch: the drivers' loops over disorder samples, sectors
// and twists.  starts (host, the runs one after another: rows values each, 2
// rows for complex operators; empty for seeded starts seed + b); evecs (host)
// receives the normalised Ritz vectors in the same layout; returns E0 per run.
inline std::vector<double> lanczos_batch(const std::vector<Hubbard*>& ops, int steps,
                                         const std::vector<double>& starts, std::vector<double>& evecs,
                                         uint64_t seed = 0) {
    const int n = (int)ops.size();
    std::vector<ed_op*> h(n);
    size_t total = 0;
    for (int b = 0; b < n; ++b) {
        h[b] = ops[b]->handle();
        total += (size_t)ops[b]->rows() * (ed_op_is_complex(h[b]) ? 2 : 1);
    }
    ed_lanczos_cfg cfg{};
    cfg.max_steps = steps;
    cfg.mode = ED_LANCZOS_FIXED;
    cfg.ritz = ED_RITZ_STORED;
    cfg.start = starts.empty() ? ED_START_RANDOM : ED_START_USER;
    cfg.seed = seed;
    evecs.resize(total);
    std::vector<ed_lanczos_result> res(n);
    check(ed_lanczos_batch(h.data(), n, &cfg, starts.empty() ? nullptr : starts.data(), ED_MEM_HOST, evecs.data(),
                           ED_MEM_HOST, nullptr, nullptr, res.data(), nullptr),
          "ed_lanczos_batch");
    std::vector<double> e0(n);
    for (int b = 0; b < n; ++b) e0[b] = res[b].e0;
    return e0;
}

// dE0/dtheta and d2E0/dtheta2 for n operators in one batched linear-response
// launch (ed_response_batch); psis_device holds the n normalised ground states
// one after another in device memory.
inline void response_batch(const std::vector<Hubbard*>& H, const std::vector<Hubbard*>& dH,
                           const std::vector<Hubbard*>& d2H, const double* psis_device, const std::vector<double>& e0,
                           int steps, std::vector<double>& first, std::vector<double>& second) {
    const int n = (int)H.size();
    std::vector<ed_op*> h(n), d(n), d2(n);
    for (int b = 0; b < n; ++b) {
        h[b] = H[b]->handle();
        d[b] = dH[b]->handle();
        d2[b] = d2H[b]->handle();
    }
    first.assign(n, 0.0);
    second.assign(n, 0.0);
    check(ed_response_batch(h.data(), d.data(), d2.data(), n, psis_device, e0.data(), steps, first.data(),
                            second.data(), nullptr),
          "ed_response_batch");
}

// Spectra::SymEigsSolver<OpType>(op, nev, ncv) with SortRule::SmallestAlge;
// eigenvectors() is rows x nev column-major (Eigen's MatrixXd layout).
class SymEigsSolver {
public:
    enum class Info { Successful, NotComputed, NotConverging };
    SymEigsSolver(Hubbard& h, int nev, int ncv) : h_(h), nev_(nev), ncv_(ncv) {}
    void init(uint64_t seed = 0) { seed_ = seed; }
    int compute(int maxit = 1000, double tol = 1e-10) {
        ed_eigs_cfg c{nev_, ncv_, maxit, ED_START_RANDOM, tol, seed_};
        evals_.assign(nev_, 0.0);
        evecs_.assign((size_t)nev_ * h_.rows(), 0.0);
        const ed_status st = ed_eigs_lowest(h_.handle(), &c, nullptr, ED_MEM_HOST, evals_.data(), evecs_.data(),
                                            ED_MEM_HOST, nullptr, &result, nullptr);
        if (st != ED_OK && st != ED_ERR_NOT_CONVERGED) check(st, "ed_eigs_lowest");
        info_ = st == ED_OK ? Info::Successful : Info::NotConverging;
        return result.nconv;
    }
    Info info() const { return info_; }
    const std::vector<double>& eigenvalues() const { return evals_; }
    const std::vector<double>& eigenvectors() const { return evecs_; }
    ed_eigs_result result{};

private:
    Hubbard& h_;
    int nev_, ncv_;
    uint64_t seed_ = 0;
    Info info_ = Info::NotComputed;
    std::vector<double> evals_, evecs_;
};

// Krylov<double>: phi0, phi are device arrays of rows() complex values
// (interleaved re, im).  Krylov_time_evol ADDS exp(-i H dt) phi0 into phi, as
// the reference's does; the Lanczos recurrence runs inside each call.
class Krylov {
public:
    int max_steps = 1000;
    double tol = 1e-10;  // stop at b < tol * |phi0|
    ed_krylov_result result{};
    Krylov(int64_t /*dimUP*/ = 0, int64_t /*dimDN*/ = 0) {}
    // The Krylov dimension of phi0 (a recurrence with no output times).
    void Make_tridiagonal_eigen(Hubbard& h, const double* phi0_dev, void* stream = nullptr) {
        ed_krylov_cfg c{max_steps, 0, tol, 0, 0};
        check(ed_krylov_evolve(h.handle(), &c, phi0_dev, ED_MEM_DEVICE, 0, nullptr, nullptr, ED_MEM_DEVICE, &result,
                               stream),
              "ed_krylov_evolve");
    }
    // phi += exp(-i H dt) phi0
    void Krylov_time_evol(Hubbard& h, const double* phi0_dev, double* phi_dev, double dt, void* stream = nullptr) {
        ed_krylov_cfg c{max_steps, 0, tol, 1, 0};
        check(ed_krylov_evolve(h.handle(), &c, phi0_dev, ED_MEM_DEVICE, 1, &dt, phi_dev, ED_MEM_DEVICE, &result,
                               stream),
              "ed_krylov_evolve");
    }
};

}  // namespace ed
