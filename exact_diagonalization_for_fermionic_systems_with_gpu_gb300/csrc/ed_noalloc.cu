// ed_noalloc.cu — y = H x without any device allocation.
//
// ed_op_perform(..., ED_MEM_DEVICE) keeps its int64 copy of x on the operator
// and allocates it with cudaMalloc on first use.  Some callers cannot let a
// library allocate device memory: code whose GPU memory is owned by another
// allocator (a framework's caching pool that has already reserved the device),
// and loops that must not pay the implicit device synchronisation a
// cudaMalloc/cudaFree can cause.  For them ed_op_perform_noalloc takes its
// scratch from the file-scope array below instead.
//
// Scratch: kNoAllocMaxElems int64 values (16 MiB) plus two ints, resident on
// a GPU from the first call on it until the process exits.  Under CUDA's
// lazy module loading the array's module is loaded, and its 16 MiB reserved,
// when the first call resolves the array's address: a caller whose allocator
// will reserve the whole device makes that first call before it does (an
// out-of-memory failure there returns ED_ERR_ALLOC).  Operators with more than
// kNoAllocMaxElems stored values (rows, or 2*rows when complex) are rejected
// with ED_ERR_RANGE.  Non-finite input is not detected here (the flag word is
// shared and cleared by the next call): y is undefined for such x.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/ed_hubbard.h"
#include "ed_internal.hpp"

namespace {

constexpr int64_t kNoAllocMaxElems = int64_t(1) << 21;
constexpr int kMaxDevices = 64;

// Device-side scratch.  In host code these names are only stand-ins: the
// device addresses come from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) int64_t g_noalloc_xq[kNoAllocMaxElems + 2];  // + padding read by row copies
static __device__ __align__(256) int g_noalloc_words[2];  // [0] max exponent, [1] non-finite flag

struct Resolved {
    int64_t* xq = nullptr;
    int* words = nullptr;
    bool ready = false;
};

Resolved g_resolved[kMaxDevices];
std::mutex g_mu;

// Resolve the scratch addresses for `device`, which must be current.
ed_status resolve(int device, Resolved* out) {
    if (device < 0 || device >= kMaxDevices) return ED_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_mu);
    Resolved& r = g_resolved[device];
    if (!r.ready) {
        void* p = nullptr;
        void* q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_xq);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&q, g_noalloc_words);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return e == cudaErrorMemoryAllocation ? ED_ERR_ALLOC : ED_ERR_CUDA;
        }
        r.xq = static_cast<int64_t*>(p);
        r.words = static_cast<int*>(q);
        r.ready = true;
    }
    *out = r;
    return ED_OK;
}

}  // namespace

extern "C" ed_status ed_op_perform_noalloc(ed_op* op, const double* x, double* y, void* stream) {
    if (!op || !x || !y) return ED_ERR_ARG;
    const int64_t n = op->D * (op->cplx ? 2 : 1);
    if (n > kNoAllocMaxElems) return ED_ERR_RANGE;
    if (cudaSetDevice(op->device) != cudaSuccess) return ED_ERR_CUDA;
    Resolved r;
    const ed_status st = resolve(op->device, &r);
    if (st != ED_OK) return st;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // launch_emax zeroes both words before the reduction, so nothing from the
    // previous call leaks into this one
    if (ed::launch_emax(x, n, r.words, r.words + 1, s) != cudaSuccess) return ED_ERR_CUDA;
    if (ed::launch_to_fx(x, n, r.words, r.xq, s) != cudaSuccess) return ED_ERR_CUDA;
    if (ed::launch_matvec_f64(op, r.xq, r.words, y, s) != cudaSuccess) return ED_ERR_CUDA;
    return ED_OK;
}
