// Arithmetic-pipe throughput probe for the Hubbard matvec design.
//
// The spin-split matvec adds ~2(n_up + n_dn) signed neighbour values per
// output element.  Whether those adds run on the FP64 pipe or on the integer
// pipes decides the whole kernel design, so this probe measures, on the GPU
// it runs on, the sustained rate of:
//   dfma   FP64 fused multiply-add              (2 flop each)
//   dadd   FP64 add
//   i64add 64-bit integer add (two 32-bit ops with carry)
//   mul64hi  high 64 bits of a signed 64x64 product (fixed-point scaling)
//   ffma   FP32 fused multiply-add              (2 flop each)
// Each thread runs 8 independent dependency chains so the pipes, not latency,
// bind.  Results print as one JSON line (ops/s; one op = one instruction of
// the named kind, not flops).
//
// Build/run:  nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o arith_probe arith_probe.cu && ./arith_probe
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { \
    fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); return 1; } } while (0)

constexpr int CHAINS = 8;

__global__ void k_dfma(double* out, double a, double b, int iters) {
    double v[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) v[c] = threadIdx.x * 1e-9 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) v[c] = fma(v[c], a, b);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += v[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_dadd(double* out, double a, double b, int iters) {
    double v[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) v[c] = threadIdx.x * 1e-9 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) v[c] = v[c] + ((c & 1) ? a : b);
    }
    double s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += v[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_i64add(long long* out, long long a, long long b, int iters) {
    long long v[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) v[c] = (long long)threadIdx.x * 77 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) v[c] = v[c] + ((c & 1) ? a : b);
    }
    long long s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s ^= v[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_mul64hi(long long* out, long long a, long long b, int iters) {
    long long v[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) v[c] = (long long)threadIdx.x * 77 + c + b;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) v[c] = __mul64hi(v[c], a) + b;
    }
    long long s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s ^= v[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_ffma(float* out, float a, float b, int iters) {
    float v[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) v[c] = threadIdx.x * 1e-6f + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) v[c] = fmaf(v[c], a, b);
    }
    float s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += v[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename F>
static float time_kernel(F launch, int reps) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0); cudaEventCreate(&e1);
    launch();  // warm-up
    cudaDeviceSynchronize();
    cudaEventRecord(e0);
    for (int r = 0; r < reps; ++r) launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0; cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    return ms / reps;
}

int main() {
    int dev = 0; cudaDeviceProp p; CK(cudaGetDeviceProperties(&p, dev));
    const int blocks = p.multiProcessorCount * 8, threads = 256;
    const size_t n = (size_t)blocks * threads;
    void* buf; CK(cudaMalloc(&buf, n * 8));
    const int it_fp64 = 512, it_int = 4096;
    double ops_fp64 = (double)n * CHAINS * it_fp64;
    double ops_int = (double)n * CHAINS * it_int;

    float t_dfma = time_kernel([&] { k_dfma<<<blocks, threads>>>((double*)buf, 0.999999, 1e-7, it_fp64); }, 3);
    float t_dadd = time_kernel([&] { k_dadd<<<blocks, threads>>>((double*)buf, 1e-7, -1e-7, it_fp64); }, 3);
    float t_i64 = time_kernel([&] { k_i64add<<<blocks, threads>>>((long long*)buf, 3, -5, it_int); }, 3);
    float t_mhi = time_kernel([&] { k_mul64hi<<<blocks, threads>>>((long long*)buf, 0x123456789abcdefLL, 7, it_int / 4); }, 3);
    float t_ffma = time_kernel([&] { k_ffma<<<blocks, threads>>>((float*)buf, 0.9999f, 1e-6f, it_int); }, 3);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    printf("{\"gpu\": \"%s\", \"sms\": %d, \"dfma_per_s\": %.4e, \"dadd_per_s\": %.4e, "
           "\"i64add_per_s\": %.4e, \"mul64hi_per_s\": %.4e, \"ffma_per_s\": %.4e, "
           "\"fp64_tflops\": %.3f, \"fp32_tflops\": %.3f}\n",
           p.name, p.multiProcessorCount,
           ops_fp64 / (t_dfma * 1e-3), ops_fp64 / (t_dadd * 1e-3),
           ops_int / (t_i64 * 1e-3), ops_int / 4 / (t_mhi * 1e-3), ops_int / (t_ffma * 1e-3),
           2 * ops_fp64 / (t_dfma * 1e-3) * 1e-12, 2 * ops_int / (t_ffma * 1e-3) * 1e-12);
    cudaFree(buf);
    return 0;
}
