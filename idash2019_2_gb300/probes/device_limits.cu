// Measures the two limits the scoring kernels are designed against:
//  * integer throughput of one GPU: IMAD (32-bit multiply-add mod 2^32, the
//    scoring kernels' inner operation), IADD3, and mma.sync s8 m16n8k32
//    (the int8 tensor path, for comparison);
//  * host <-> device bandwidth from page-locked memory: copy engines in each
//    direction, both directions at once, and kernels loading / storing
//    through mapped page-locked memory.
// Every access stays inside its allocation; nothing waits on another thread.
// Build and run:
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o _build/device_limits \
//        idash2019_2_gb300/probes/device_limits.cu && ./_build/device_limits
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>

#define CK(x)                                                                     \
    do {                                                                          \
        cudaError_t e_ = (x);                                                     \
        if (e_ != cudaSuccess) {                                                  \
            std::printf("error %s at line %d\n", cudaGetErrorString(e_), __LINE__); \
            return 1;                                                             \
        }                                                                         \
    } while (0)

// 8 independent dependency chains per thread, 16 unrolled steps each.
__global__ void k_imad(uint32_t *out, uint32_t seed, int iters) {
    uint32_t a0 = threadIdx.x ^ seed, a1 = a0 * 3u, a2 = a0 * 5u, a3 = a0 * 7u;
    uint32_t a4 = a0 + 1, a5 = a0 + 2, a6 = a0 + 3, a7 = a0 + 4;
    const uint32_t w = seed | 1u;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = a0 * w + a1; a1 = a1 * w + a2; a2 = a2 * w + a3; a3 = a3 * w + a4;
            a4 = a4 * w + a5; a5 = a5 * w + a6; a6 = a6 * w + a7; a7 = a7 * w + a0;
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
}

__global__ void k_iadd3(uint32_t *out, uint32_t seed, int iters) {
    uint32_t a0 = threadIdx.x ^ seed, a1 = a0 * 3u, a2 = a0 * 5u, a3 = a0 * 7u;
    uint32_t a4 = a0 + 1, a5 = a0 + 2, a6 = a0 + 3, a7 = a0 + 4;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = a0 + a1 + seed; a1 = a1 + a2 + seed; a2 = a2 + a3 + seed; a3 = a3 + a4 + seed;
            a4 = a4 + a5 + seed; a5 = a5 + a6 + seed; a6 = a6 + a7 + seed; a7 = a7 + a0 + seed;
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
}

// 4 independent accumulator tiles per warp.
__global__ void k_mma_s8(uint32_t *out, uint32_t seed, int iters) {
    const uint32_t a[4] = {seed, seed * 3u, seed * 5u, seed * 7u}, b[2] = {seed * 11u, seed * 13u};
    int32_t c[4][4] = {};
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
#pragma unroll
            for (int t = 0; t < 4; ++t)
                asm volatile(
                    "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};"
                    : "+r"(c[t][0]), "+r"(c[t][1]), "+r"(c[t][2]), "+r"(c[t][3])
                    : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
        }
    }
    uint32_t x = 0;
    for (int t = 0; t < 4; ++t) x ^= c[t][0] ^ c[t][1] ^ c[t][2] ^ c[t][3];
    out[blockIdx.x * blockDim.x + threadIdx.x] = x;
}

__global__ void k_copy16(const int4 *__restrict__ src, int4 *dst, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

static int integer_throughput(const cudaDeviceProp &p, double sm_hz) {
    const int blocks = p.multiProcessorCount * 8, threads = 256;
    uint32_t *d = nullptr;
    CK(cudaMalloc(&d, sizeof(uint32_t) * blocks * threads));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const int iters = 4096, mma_iters = 1024;
    const double ops = (double)blocks * threads * iters * 16 * 8;
    const double macs = (double)blocks * (threads / 32) * mma_iters * 16 * (16.0 * 8 * 32);
    for (int rep = 0; rep < 2; ++rep) {
        float ms = 0;
        CK(cudaEventRecord(e0));
        k_imad<<<blocks, threads>>>(d, 12345u, iters);
        CK(cudaEventRecord(e1));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        std::printf("IMAD: %.3f ms  %.2f T/s  %.1f per clock per SM\n", ms, ops / ms / 1e9,
                    ops / (ms * 1e-3) / p.multiProcessorCount / sm_hz);
        CK(cudaEventRecord(e0));
        k_iadd3<<<blocks, threads>>>(d, 12345u, iters);
        CK(cudaEventRecord(e1));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        std::printf("IADD3: %.3f ms  %.2f T/s  %.1f per clock per SM\n", ms, ops / ms / 1e9,
                    ops / (ms * 1e-3) / p.multiProcessorCount / sm_hz);
        CK(cudaEventRecord(e0));
        k_mma_s8<<<blocks, threads>>>(d, 12345u, mma_iters);
        CK(cudaEventRecord(e1));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        std::printf("mma.sync s8 m16n8k32: %.3f ms  %.2f T MAC/s\n", ms, macs / ms / 1e9);
    }
    CK(cudaGetLastError());
    CK(cudaFree(d));
    return 0;
}

static int host_link(const cudaDeviceProp &p) {
    const size_t big = 2ull << 30, small = 400ull << 20;
    void *h_out = nullptr, *h_in = nullptr, *d_out = nullptr, *d_in = nullptr;
    CK(cudaMallocHost(&h_out, big));
    CK(cudaMallocHost(&h_in, small));
    CK(cudaMalloc(&d_out, big));
    CK(cudaMalloc(&d_in, small));
    CK(cudaMemset(d_out, 1, big));
    CK(cudaMemset(d_in, 2, small));
    std::memset(h_out, 0, big);
    std::memset(h_in, 3, small);
    cudaStream_t s[4];
    for (auto &x : s) CK(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    void *h_out_dev = nullptr, *h_in_dev = nullptr;
    CK(cudaHostGetDevicePointer(&h_out_dev, h_out, 0));
    CK(cudaHostGetDevicePointer(&h_in_dev, h_in, 0));
    float ms = 0;
    for (int rep = 0; rep < 2; ++rep) {
        CK(cudaEventRecord(e0, s[0]));
        CK(cudaMemcpyAsync(h_out, d_out, big, cudaMemcpyDeviceToHost, s[0]));
        CK(cudaEventRecord(e1, s[0]));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        std::printf("D2H copy 2 GiB: %.2f ms %.1f GB/s\n", ms, big / ms / 1e6);
        CK(cudaEventRecord(e0, s[0]));
        CK(cudaMemcpyAsync(d_in, h_in, small, cudaMemcpyHostToDevice, s[0]));
        CK(cudaEventRecord(e1, s[0]));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        std::printf("H2D copy 400 MiB: %.2f ms %.1f GB/s\n", ms, small / ms / 1e6);

        CK(cudaDeviceSynchronize());
        CK(cudaEventRecord(e0, 0));
        for (int c = 0; c < 8; ++c)
            CK(cudaMemcpyAsync((char *)h_out + c * (big / 8), (char *)d_out + c * (big / 8), big / 8,
                               cudaMemcpyDeviceToHost, s[c % 4]));
        CK(cudaDeviceSynchronize());
        CK(cudaEventRecord(e1, 0));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        std::printf("D2H 8 copies on 4 streams: %.2f ms %.1f GB/s\n", ms, big / ms / 1e6);

        CK(cudaDeviceSynchronize());
        CK(cudaEventRecord(e0, 0));
        CK(cudaMemcpyAsync(d_in, h_in, small, cudaMemcpyHostToDevice, s[1]));
        CK(cudaMemcpyAsync(h_out, d_out, big, cudaMemcpyDeviceToHost, s[2]));
        CK(cudaDeviceSynchronize());
        CK(cudaEventRecord(e1, 0));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        std::printf("H2D 400 MiB and D2H 2 GiB at once: %.2f ms %.1f GB/s total\n", ms, (big + small) / ms / 1e6);

        CK(cudaEventRecord(e0, s[0]));
        k_copy16<<<p.multiProcessorCount * 8, 512, 0, s[0]>>>((const int4 *)d_out, (int4 *)h_out_dev, big / 16);
        CK(cudaEventRecord(e1, s[0]));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        std::printf("kernel stores to mapped host 2 GiB: %.2f ms %.1f GB/s\n", ms, big / ms / 1e6);
        CK(cudaEventRecord(e0, s[0]));
        k_copy16<<<p.multiProcessorCount * 8, 512, 0, s[0]>>>((const int4 *)h_in_dev, (int4 *)d_in, small / 16);
        CK(cudaEventRecord(e1, s[0]));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(&ms, e0, e1));
        std::printf("kernel loads from mapped host 400 MiB: %.2f ms %.1f GB/s\n", ms, small / ms / 1e6);
    }
    CK(cudaGetLastError());
    for (auto &x : s) CK(cudaStreamDestroy(x));
    CK(cudaFreeHost(h_out));
    CK(cudaFreeHost(h_in));
    CK(cudaFree(d_out));
    CK(cudaFree(d_in));
    return 0;
}

int main() {
    cudaDeviceProp p{};
    CK(cudaGetDeviceProperties(&p, 0));
    int khz = 0;
    CK(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, 0));
    std::printf("%s: %d SMs, compute capability %d.%d, max SM clock %d MHz\n", p.name, p.multiProcessorCount, p.major,
                p.minor, khz / 1000);
    if (integer_throughput(p, khz * 1e3)) return 1;
    return host_link(p);
}
