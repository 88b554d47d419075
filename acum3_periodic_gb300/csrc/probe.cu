// probe.cu -- measures the FP32 and FP64 FMA throughput of the device (the CUDA-core
// peaks the tonal kernels are compute-bound against), with CUDA events; a self-test of
// the bounded barrier wait that every pipelined kernel uses; and a self-test of the
// shared-memory to tensor-memory copy and the tensor-memory loads of the record stages.
#include <cuda_runtime.h>

#include "acum_internal.h"
#include "ptx.h"

namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_chains(T* out, int iters, T b, T c)
{
    // 8 independent dependency chains per thread keep the FMA pipe busy
    T a0 = (T)threadIdx.x, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
      a7 = a0 + 7;
    for (int i = 0; i < iters; ++i) {
        a0 = a0 * b + c; a1 = a1 * b + c; a2 = a2 * b + c; a3 = a3 * b + c;
        a4 = a4 * b + c; a5 = a5 * b + c; a6 = a6 * b + c; a7 = a7 * b + c;
    }
    const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == (T)-12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
cudaError_t measure(int sms, int iters, double* tflops)
{
    T* out = nullptr;
    cudaError_t e = cudaMalloc(&out, sizeof(T) * 256 * sms * 8);
    if (e != cudaSuccess) return e;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 8;
    fma_chains<T><<<blocks, 256>>>(out, iters / 10, (T)0.999999, (T)1e-7);  // warm-up
    cudaEventRecord(a);
    fma_chains<T><<<blocks, 256>>>(out, iters, (T)0.999999, (T)1e-7);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess) return e;
    const double flops = 2.0 * 8.0 * (double)iters * blocks * 256.0;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return cudaGetLastError();
}

// One block waits on an mbarrier whose phase is completed (arrive = 1) or never completed
// (arrive = 0) with the bounded wait of the kernels; reports whether it gave up and how
// long it waited.
__global__ void wait_selftest_kernel(unsigned long long limit_ns, int arrive, int* timed_out,
                                     unsigned long long* waited_ns)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        acum::mbar_init(&bar, 1);
        acum::mbar_fence_init();
    }
    __syncthreads();
    if (arrive && threadIdx.x == 0) acum::mbar_arrive(&bar);
    __syncthreads();
    const unsigned long long t0 = acum::global_ns();
    const bool ok = acum::mbar_wait_bounded(&bar, 0u, limit_ns);
    const unsigned long long dt = acum::global_ns() - t0;
    if (threadIdx.x == 0) {
        *timed_out = ok ? 0 : 1;
        *waited_ns = dt;
    }
}

// Tensor-memory path of the record stages: a pattern laid out like one element-pair tile
// (10 blocks of 32 rows x 16 bytes) is copied from shared memory into TMEM by ten
// 32x128b.warpx4 copies, read back by all 16 warps (each from its lane quarter) with one
// 32-column and one 8-column load, and compared.  Warps 0-3 also write what they read.
constexpr int kTmemPatWords = 10 * 32 * 4;
constexpr int kTmemProbeSmem = 64 * 1024;  // the pattern, then a margin of unused words

__global__ void __launch_bounds__(512, 1) tmem_selftest_kernel(int* mismatches, unsigned* readback, int* timed_out)
{
    extern __shared__ __align__(1024) unsigned char tsm[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t taddr_s;
    unsigned* pat = reinterpret_cast<unsigned*>(tsm);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kTmemProbeSmem / 4; i += blockDim.x) pat[i] = i < kTmemPatWords ? 0x10000u + i : 0u;
    if (threadIdx.x == 0) {
        acum::mbar_init(&bar, 1);
        acum::mbar_fence_init();
    }
    if (warp == 0) {
        acum::tmem_alloc(&taddr_s, 64);
        acum::tmem_relinquish();
    }
    acum::fence_proxy_async_smem();
    acum::tmem_fence_before();
    __syncthreads();
    acum::tmem_fence_after();
    const uint32_t tbase = taddr_s;
    if (threadIdx.x == 0) {
        for (int c = 0; c < 10; ++c)
            acum::tmem_cp_32x128b_warpx4(tbase + 4u * c, acum::smem_desc_plain(pat + c * 128, 128, 128));
        acum::tmem_commit(&bar);
    }
    const bool ok = acum::mbar_wait_bounded(&bar, 0u);
    acum::tmem_fence_after();
    uint32_t r[40];
    if (__all_sync(0xffffffffu, ok)) {
        const uint32_t t = tbase + ((uint32_t)(32 * (warp & 3)) << 16);
        acum::tmem_ld32(t, r);
        acum::tmem_ld8(t + 32u, r);
        acum::tmem_wait_ld(r);
        int bad = 0;
#pragma unroll
        for (int j = 0; j < 40; ++j) bad += r[j] != 0x10000u + (unsigned)((j >> 2) * 128 + lane * 4 + (j & 3)) ? 1 : 0;
        if (bad) atomicAdd(mismatches, bad);
        if (warp < 4)
            for (int j = 0; j < 40; ++j) readback[(warp * 32 + lane) * 40 + j] = r[j];
    } else if (threadIdx.x == 0) {
        *timed_out = 1;
    }
    acum::tmem_fence_before();
    __syncthreads();
    if (warp == 0) acum::tmem_dealloc(tbase, 64);
}

}  // namespace

extern "C" int acum_selftest_tmem(int device, int* mismatches, unsigned* readback)
{
    if (!mismatches) return ACUM_ERR_INVALID;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return ACUM_ERR_CUDA;
    int* d_mis = nullptr;
    unsigned* d_rb = nullptr;
    cudaError_t e = cudaMalloc(&d_mis, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&d_rb, 4 * 32 * 40 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(d_mis, 0, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(d_rb, 0, 4 * 32 * 40 * sizeof(unsigned));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(tmem_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTmemProbeSmem);
    if (e == cudaSuccess) {
        tmem_selftest_kernel<<<1, 512, kTmemProbeSmem>>>(d_mis, d_rb, d_mis + 1);
        e = cudaDeviceSynchronize();
    }
    int h[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, d_mis, sizeof(h), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && readback)
        e = cudaMemcpy(readback, d_rb, 4 * 32 * 40 * sizeof(unsigned), cudaMemcpyDeviceToHost);
    if (d_mis) cudaFree(d_mis);
    if (d_rb) cudaFree(d_rb);
    cudaSetDevice(prev);
    if (e != cudaSuccess) return ACUM_ERR_CUDA;
    *mismatches = h[1] ? -1 : h[0];
    return ACUM_OK;
}

extern "C" int acum_selftest_wait(int device, double limit_s, int arrive, int* timed_out, double* waited_s)
{
    if (!timed_out || !waited_s || !(limit_s > 0.0) || limit_s > 10.0) return ACUM_ERR_INVALID;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return ACUM_ERR_CUDA;
    int* d_to = nullptr;
    unsigned long long* d_ns = nullptr;
    cudaError_t e = cudaMalloc(&d_to, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&d_ns, sizeof(unsigned long long));
    if (e == cudaSuccess) {
        wait_selftest_kernel<<<1, 32>>>((unsigned long long)(limit_s * 1e9), arrive ? 1 : 0, d_to, d_ns);
        e = cudaDeviceSynchronize();
    }
    unsigned long long ns = 0;
    if (e == cudaSuccess) e = cudaMemcpy(timed_out, d_to, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&ns, d_ns, sizeof(ns), cudaMemcpyDeviceToHost);
    if (d_to) cudaFree(d_to);
    if (d_ns) cudaFree(d_ns);
    cudaSetDevice(prev);
    *waited_s = ns * 1e-9;
    return e == cudaSuccess ? ACUM_OK : ACUM_ERR_CUDA;
}

extern "C" int acum_measure_peak(int device, int which, double* tflops)
{
    if (!tflops || which < 0 || which > 1) return ACUM_ERR_INVALID;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return ACUM_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaError_t e = which == 0 ? measure<float>(sms, 1 << 12, tflops) : measure<double>(sms, 1 << 7, tflops);
    cudaSetDevice(prev);
    return e == cudaSuccess ? ACUM_OK : ACUM_ERR_CUDA;
}
