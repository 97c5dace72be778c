// ed_matvec_common.cuh — pieces shared by the matvec kernels.
#pragma once

#include "ed_device.cuh"
#include "ed_internal.hpp"
#include "ed_lanczos.hpp"
#include "ed_lanczos_dev.cuh"

namespace ed {
using namespace dev;

__device__ __forceinline__ int64_t apply_sign(int64_t v, uint32_t e) {
    int64_t m = (int64_t)((int32_t)e >> 31);  // 0 or -1
    return (v ^ m) - m;
}

template <bool CPLX>
__device__ __forceinline__ void apply_class(i128& ar, i128& ai, int64_t sr, int64_t si,
                                            const int64_t* __restrict__ coef, int c, bool unit, int Fc) {
    if (unit) {
        ar += ((i128)sr) << Fc;
        if (CPLX) ai += ((i128)si) << Fc;
        return;
    }
    const int64_t cr = coef[2 * c];
    ar += mul_wide(sr, cr);
    if (CPLX) {
        const int64_t ci = coef[2 * c + 1];
        ai += mul_wide(si, cr);
        if (ci != 0) {
            ar -= mul_wide(si, ci);
            ai += mul_wide(sr, ci);
        }
    }
}

// Element (row, col) pair of the up term: x[(uoff + d) * W]; uoff = col * dimDN
// is a 32-bit element offset (the whole vector has < 2^32 elements), so the
// address is one wide multiply-add.
template <bool CPLX>
__device__ __forceinline__ void load_x(const int64_t* __restrict__ xq, uint32_t idx, int64_t& r, int64_t& i) {
    if (CPLX) {
        const longlong2 v = __ldg(reinterpret_cast<const longlong2*>(xq) + idx);
        r = v.x;
        i = v.y;
    } else {
        r = __ldg(xq + idx);
        i = 0;
    }
}

// Lanczos epilogue of a matvec launch: block sums of <x, u> and max|u|,
// then the last block finishes the grid reduction and the step scalars.
__device__ __forceinline__ void mv_lanczos_epilogue(const MvArgs& a, i128 dot, uint64_t mx, int s_u) {
    __shared__ i128 s128[32];
    __shared__ uint64_t s64[32];
    LzState* lz = reinterpret_cast<LzState*>(a.lz);
    const i128 bs = block_sum_i128(dot, s128);
    const uint64_t bm = block_max_u64(mx, s64);
    if (threadIdx.x == 0) {
        lz->part_lo[blockIdx.x] = (uint64_t)bs;
        lz->part_hi[blockIdx.x] = (uint64_t)((u128)bs >> 64);
        lz->part_max[blockIdx.x] = bm;
    }
    if (elect_last_block(&lz->counter[0])) {
        i128 s = 0;
        uint64_t m = 0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
            s += (i128)(((u128)__ldcg(lz->part_hi + i) << 64) | __ldcg(lz->part_lo + i));
            const uint64_t pm = __ldcg(lz->part_max + i);
            m = pm > m ? pm : m;
        }
        s = block_sum_i128(s, s128);
        m = block_max_u64(m, s64);
        if (threadIdx.x == 0) {
            lz_after_matvec(lz, a.step, s, m, s_u, a.Fc);
            lz->counter[0] = 0;
        }
    }
}

}  // namespace ed
