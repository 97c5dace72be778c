// ed_device.cuh — device helpers shared by the Hubbard kernels.
//
// Number format ("FX"): a vector is an int64 array q with one exponent e per
// vector, value_i = q_i * 2^e.  On this GPU the FP64 pipe issues ~1/64 of the
// FP32 rate (measured 0.5e12 DFMA/s on GB300), while 64-bit integer adds run
// on the integer pipes at tens of times that rate.  The matvec therefore sums
// +-neighbour values exactly in int64 and applies each real coefficient once
// per (row, coefficient class) with a 64x64->128-bit product; reductions are
// exact 128-bit integer sums, so they are also independent of the order in
// which blocks finish.
//
// Conversions between FP64 and FX are done with integer bit manipulation of
// the IEEE-754 encoding (sign | 11-bit biased exponent | 52-bit fraction),
// never through the FP64 pipe.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ed {
namespace dev {

typedef __int128 i128;
typedef unsigned __int128 u128;

// ---------------------------------------------------------------- FP64 bits --

// Biased exponent field of |v| (0 for zero/subnormal, 2047 for Inf/NaN).
__device__ __forceinline__ int f64_biased_exp(double v) {
    return (int)((__double_as_longlong(v) >> 52) & 0x7FF);
}

// Exponent E of the FX scale for a vector whose largest biased exponent is
// emax: |q| < 2^54 for every element.
__host__ __device__ __forceinline__ int fx_exp_from_emax(int emax) { return emax - 1076; }

// q = round(v * 2^-E), ties away from zero.  Requires |v| * 2^-E < 2^63.
__device__ __forceinline__ int64_t f64_to_fx(double v, int E) {
    long long bits = __double_as_longlong(v);
    int be = (int)((bits >> 52) & 0x7FF);
    uint64_t m = (uint64_t)bits & 0x000FFFFFFFFFFFFFULL;
    int ex;
    if (be == 0) {
        ex = -1074;
    } else {
        m |= 0x0010000000000000ULL;
        ex = be - 1075;
    }
    int sh = ex - E;
    uint64_t q;
    if (sh >= 0) {
        q = (sh >= 63) ? 0 : (m << sh);
    } else {
        int r = -sh;
        q = (r >= 64) ? 0 : ((m + (1ULL << (r - 1))) >> r);
    }
    return bits < 0 ? -(int64_t)q : (int64_t)q;
}

// Round a non-zero unsigned magnitude mag * 2^E to the nearest double
// (ties to even) and attach the sign.  Normal range only; results below the
// normal range go through a slower exact path.
__device__ __forceinline__ double u128_to_f64(u128 mag, int E, bool neg) {
    if (mag == 0) return neg ? -0.0 : 0.0;
    uint64_t hi = (uint64_t)(mag >> 64), lo = (uint64_t)mag;
    int msb = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
    uint64_t M;
    int exp2;
    if (msb > 52) {
        int s = msb - 52;
        u128 q = mag >> s;
        u128 rem = mag - (q << s);
        u128 half = ((u128)1) << (s - 1);
        M = (uint64_t)q;
        if (rem > half || (rem == half && (M & 1ULL))) ++M;
        exp2 = s + E;
        if (M == (1ULL << 53)) { M >>= 1; ++exp2; }
    } else {
        M = lo << (52 - msb);
        exp2 = E - (52 - msb);
    }
    int be = exp2 + 1075;  // M in [2^52, 2^53): value = M * 2^exp2
    if (be >= 2047) return neg ? -INFINITY : INFINITY;
    if (be <= 0) {
        // Below the normal range (rare): scale exactly into range, then let
        // one final multiply by 2^-600 do the single rounding.
        if (exp2 < -1622) return neg ? -0.0 : 0.0;
        double r = __ull2double_rn(M);  // exact, M < 2^53
        r = r * __longlong_as_double((long long)(exp2 + 600 + 1023) << 52);
        r = r * 0x1p-600;
        return neg ? -r : r;
    }
    long long bits = ((long long)be << 52) | (long long)(M & 0x000FFFFFFFFFFFFFULL);
    if (neg) bits |= (long long)0x8000000000000000ULL;
    return __longlong_as_double(bits);
}

__device__ __forceinline__ double i128_to_f64(i128 v, int E) {
    bool neg = v < 0;
    u128 mag = neg ? (u128)(-v) : (u128)v;
    return u128_to_f64(mag, E, neg);
}

__device__ __forceinline__ double i64_to_f64(int64_t v, int E) {
    bool neg = v < 0;
    u128 mag = neg ? (u128)(uint64_t)(-(v + 1)) + 1 : (u128)(uint64_t)v;
    return u128_to_f64(mag, E, neg);
}

// Signed 64x64 -> 128-bit product.
__device__ __forceinline__ i128 mul_wide(int64_t a, int64_t b) {
    uint64_t lo = (uint64_t)a * (uint64_t)b;
    int64_t hi = __mul64hi(a, b);
    return (i128)(((u128)(uint64_t)hi << 64) | (u128)lo);
}

// round(v / 2^s), ties toward +inf, s >= 0.
__device__ __forceinline__ i128 shr_round(i128 v, int s) {
    if (s <= 0) return v;
    return (v + ((i128)1 << (s - 1))) >> s;
}

// round(v / 2^s) as int64 for a (warp-uniform) s >= 0 when the result is
// known to fit in 64 bits: one 128-bit add and a funnel shift.
__device__ __forceinline__ int64_t shr_round_i64(i128 v, int s) {
    if (s <= 0) return (int64_t)v;
    if (s < 64) {
        const u128 t = (u128)v + ((u128)1 << (s - 1));
        const uint64_t lo = (uint64_t)t, hi = (uint64_t)(t >> 64);
        return (int64_t)((lo >> s) | (hi << (64 - s)));
    }
    return (int64_t)((v + ((i128)1 << (s - 1))) >> s);
}

__device__ __forceinline__ int bitlen_u64(uint64_t v) { return v ? 64 - __clzll((long long)v) : 0; }

// ---------------------------------------------------------- warp / block ops --

__device__ __forceinline__ i128 warp_sum_i128(i128 v) {
    uint64_t lo = (uint64_t)v, hi = (uint64_t)((u128)v >> 64);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        uint64_t olo = __shfl_down_sync(0xffffffffu, lo, off);
        uint64_t ohi = __shfl_down_sync(0xffffffffu, hi, off);
        uint64_t nlo = lo + olo;
        hi = hi + ohi + (nlo < lo ? 1ULL : 0ULL);
        lo = nlo;
    }
    return (i128)(((u128)hi << 64) | lo);
}

__device__ __forceinline__ uint64_t warp_max_u64(uint64_t v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        uint64_t o = __shfl_down_sync(0xffffffffu, v, off);
        v = o > v ? o : v;
    }
    return v;
}

__device__ __forceinline__ int warp_max_int(int v) { return __reduce_max_sync(0xffffffffu, v); }

// Block-wide reductions; the result is valid in thread 0.  `scratch` needs
// 32 entries of the value type; blockDim.x must be a multiple of 32.
__device__ __forceinline__ i128 block_sum_i128(i128 v, i128* scratch) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum_i128(v);
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    i128 r = 0;
    if (wid == 0) {
        r = lane < nw ? scratch[lane] : (i128)0;
        r = warp_sum_i128(r);
    }
    return r;
}

// Sum and max in one pass (two barriers); results valid in thread 0.
__device__ __forceinline__ void block_sum_max(i128& v, uint64_t& m, i128* s128, uint64_t* s64) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum_i128(v);
    m = warp_max_u64(m);
    __syncthreads();
    if (lane == 0) {
        s128[wid] = v;
        s64[wid] = m;
    }
    __syncthreads();
    if (wid == 0) {
        v = lane < nw ? s128[lane] : (i128)0;
        m = lane < nw ? s64[lane] : 0ULL;
        v = warp_sum_i128(v);
        m = warp_max_u64(m);
    }
}

__device__ __forceinline__ uint64_t block_max_u64(uint64_t v, uint64_t* scratch) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_max_u64(v);
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    uint64_t r = 0;
    if (wid == 0) {
        r = lane < nw ? scratch[lane] : 0ULL;
        r = warp_max_u64(r);
    }
    return r;
}

__device__ __forceinline__ int block_max_int(int v, int* scratch) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_max_int(v);
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    int r = 0;
    if (wid == 0) {
        r = lane < nw ? scratch[lane] : 0;
        r = warp_max_int(r);
    }
    return r;
}

__device__ __forceinline__ double block_sum_f64(double v, double* scratch) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = lane < nw ? scratch[lane] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) r += __shfl_down_sync(0xffffffffu, r, off);
    }
    return r;
}

// "Last block done" election for single-pass grid reductions: every block
// publishes its partial, fences, and bumps the counter; the block that sees
// gridDim.x-1 finishes the reduction and resets the counter for reuse.
// The block's partial must have been written by thread 0 (only that thread
// fences before bumping the counter).
__device__ __forceinline__ bool elect_last_block(unsigned int* counter) {
    __shared__ bool is_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int prev = atomicAdd(counter, 1u);
        is_last = (prev == gridDim.x - 1);
        if (is_last) __threadfence();
    }
    __syncthreads();
    return is_last;
}

// ------------------------------------------------------------------- Philox --
// Philox4x64-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of two 64x64
// multiplies with the published multipliers and Weyl key increments.  The
// counter of block b is (b+1, 0, 0, 0) so that element k of the stream
// equals the k-th output of numpy.random.Philox(key=[seed, 0]).
struct Philox4 {
    uint64_t v[4];
};

__host__ __device__ __forceinline__ void mulhilo64(uint64_t a, uint64_t b, uint64_t* hi, uint64_t* lo) {
#ifdef __CUDA_ARCH__
    *lo = a * b;
    *hi = __umul64hi(a, b);
#else
    unsigned __int128 p = (unsigned __int128)a * b;
    *lo = (uint64_t)p;
    *hi = (uint64_t)(p >> 64);
#endif
}

__host__ __device__ __forceinline__ Philox4 philox4x64_10(uint64_t block, uint64_t seed) {
    const uint64_t M0 = 0xD2E7470EE14C6C93ULL, M1 = 0xCA5A826395121157ULL;
    const uint64_t W0 = 0x9E3779B97F4A7C15ULL, W1 = 0xBB67AE8584CAA73BULL;
    uint64_t c0 = block + 1, c1 = (block + 1 == 0) ? 1 : 0, c2 = 0, c3 = 0;
    uint64_t k0 = seed, k1 = 0;
    for (int r = 0; r < 10; ++r) {
        uint64_t hi0, lo0, hi1, lo1;
        mulhilo64(M0, c0, &hi0, &lo0);
        mulhilo64(M1, c2, &hi1, &lo1);
        uint64_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += W0;
        k1 += W1;
    }
    Philox4 out;
    out.v[0] = c0; out.v[1] = c1; out.v[2] = c2; out.v[3] = c3;
    return out;
}

// uniform(-1, 1) from the top 52 bits: [1,2) by exponent bits, then 2v - 3.
__host__ __device__ __forceinline__ double uniform_pm1(uint64_t r) {
    uint64_t bits = 0x3FF0000000000000ULL | (r >> 12);
    double v;
#ifdef __CUDA_ARCH__
    v = __longlong_as_double((long long)bits);
#else
    __builtin_memcpy(&v, &bits, 8);
#endif
    return 2.0 * v - 3.0;
}

}  // namespace dev
}  // namespace ed
