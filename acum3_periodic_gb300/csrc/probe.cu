// probe.cu -- measures the FP32 and FP64 FMA throughput of the device (the CUDA-core
// peaks the tonal kernels are compute-bound against), with CUDA events.
#include <cuda_runtime.h>

#include "acum_internal.h"

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

}  // namespace

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
