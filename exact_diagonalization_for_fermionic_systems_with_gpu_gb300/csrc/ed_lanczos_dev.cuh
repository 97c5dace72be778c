// ed_lanczos_dev.cuh — scalar bookkeeping of the FX Lanczos recurrence,
// run by one thread of the last block of each grid reduction.
//
// Recurrence (HubMatrix_GPU.cuh:573-582 restated on unnormalised vectors):
//   v_j = w_j / beta_j,  u = H w_j (exact integer accumulation, then >> s_u)
//   alpha_j   = <w_j, u> / beta_j^2
//   w_{j+1}   = u/beta_j - (alpha_j/beta_j) w_j - (beta_j/beta_{j-1}) w_{j-1}
//   beta_{j+1} = |w_{j+1}|
// Every vector is int64 with its own exponent; the three real multipliers of
// the axpy become int64 coefficients at[k] with per-term fractional bits so
// that |w_{j+1} q| < 2^54 by construction (room for the matvec's sums).
#pragma once

#include "ed_device.cuh"
#include "ed_lanczos.hpp"

namespace ed {
namespace dev {

// x * 2^k, exact: an add to the exponent field when x and the result are
// normal numbers, ldexp otherwise.
__device__ __forceinline__ double scale2(double x, int k) {
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7FF);
    if (ex == 0 || ex + k <= 0 || ex + k >= 0x7FF) return ldexp(x, k);
    return __longlong_as_double(b + ((long long)k << 52));
}

// The exponent frexp returns for x != 0 (|x| in [2^(e-1), 2^e)).
__device__ __forceinline__ int frexp_exp(double x) {
    const int ex = (int)((__double_as_longlong(x) >> 52) & 0x7FF);
    if (ex == 0 || ex == 0x7FF) {
        int e = 0;
        frexp(x, &e);
        return e;
    }
    return ex - 1022;
}

// Scalars of one step after the matvec reduction.
struct LzCoefs {
    double alpha;
    int64_t at[3];
    int Fa;
    int e_w;
};

// alpha_j and the integer axpy coefficients of step j from the exact
// <w_j, u> (alpha_raw), slot j (eX, mX, bj and ib = 1 / bj, computed when
// slot j was completed) and slot j-1 (eP, mP and ibP = 1 / beta_{j-1}).
__device__ inline LzCoefs lz_coefs(int j, i128 alpha_raw, int e_u, uint64_t m_u, int eX, uint64_t mX, double bj,
                                   double ib, int eP, uint64_t mP, double ibP, int status) {
    LzCoefs c;
    if (!(bj > 0.0) || status != 0) {
        // after a breakdown (or a bad start) the recurrence only carries zeros
        c.alpha = 0.0;
        for (int k = 0; k < 3; ++k) c.at[k] = 0;
        c.Fa = 0;
        c.e_w = eX;
        return c;
    }
    const double anum = i128_to_f64(alpha_raw, eX + e_u + 24);
    const double aj = (anum * ib) * ib;
    c.alpha = aj;

    double a[3];
    uint64_t mm[3];
    a[0] = scale2(ib, e_u);
    mm[0] = m_u;
    a[1] = -aj * scale2(ib, eX);
    mm[1] = mX;
    if (j > 0) {
        a[2] = -bj * scale2(ibP, eP);
        mm[2] = mP;
    } else {
        a[2] = 0.0;
        mm[2] = 0;
    }
    double B = 0.0;
    for (int k = 0; k < 3; ++k) B += fabs(a[k]) * (double)mm[k];
    B *= (1.0 + 1e-9);
    const int kB = B > 0.0 ? frexp_exp(B) : 0;  // B < 2^kB
    const int e_w = kB - 54;
    // One common number of fractional bits for the three integer
    // coefficients: the largest |a_k| 2^-e_w sets it so every |at_k| < 2^62
    // (scaling by 2^-e_w is exact, so its frexp exponent is the largest
    // exponent of the a_k minus e_w).
    int ka = 0;
    bool any = false;
    for (int k = 0; k < 3; ++k)
        if (mm[k] != 0 && a[k] != 0.0) {
            const int ek = frexp_exp(a[k]) - e_w;
            ka = any ? max(ka, ek) : ek;
            any = true;
        }
    const int Fmin = 62 - ka;
    for (int k = 0; k < 3; ++k) c.at[k] = (mm[k] != 0 && a[k] != 0.0) ? llrint(scale2(a[k], Fmin - e_w)) : 0;
    c.Fa = Fmin;
    c.e_w = e_w;
    return c;
}

// 1 / beta for the w_{j-1} coefficient (beta > 0 on every step that uses it;
// 0 keeps a breakdown's zeros finite).
__device__ inline double lz_inv(double b) { return b > 0.0 ? 1.0 / b : 0.0; }

// |w_{j+1}| from the exact sum of (q q) >> 16 at exponent e_w.
__device__ inline double lz_beta(i128 sumsq, int e_w) { return sqrt(i128_to_f64(sumsq, 2 * e_w + 16)); }

__device__ inline void lz_after_matvec(LzState* lz, int j, i128 alpha_raw, uint64_t m_u, int s_u, int Fc) {
    const int eX = lz->e[j];
    const int e_u = eX - Fc + s_u;
    lz->s_u = s_u;
    lz->e_u = e_u;
    lz->m_u = m_u;
    const LzCoefs c = lz_coefs(j, alpha_raw, e_u, m_u, eX, lz->m[j], lz->beta[j], lz_inv(lz->beta[j]),
                               j > 0 ? lz->e[j - 1] : 0,
                               j > 0 ? lz->m[j - 1] : 0, j > 0 ? lz_inv(lz->beta[j - 1]) : 0.0, lz->status);
    lz->alpha[j] = c.alpha;
    for (int k = 0; k < 3; ++k) {
        lz->at[k] = c.at[k];
        lz->sh[k] = 0;
    }
    lz->Fa = c.Fa;
    lz->e_w = c.e_w;
}

__device__ inline void lz_after_axpy(LzState* lz, int j, i128 sumsq, uint64_t m_w) {
    const int e_w = lz->e_w;
    lz->e[j + 1] = e_w;
    lz->m[j + 1] = m_w;
    lz->beta[j + 1] = lz_beta(sumsq, e_w);
    const int bits = bitlen_u64(m_w);
    if (bits < lz->min_bits) lz->min_bits = bits;
    if (m_w == 0 && lz->status == 0) lz->status = 7;  // breakdown
    lz->steps_done = j + 1;
}

}  // namespace dev
}  // namespace ed
