// peak.cu -- FMA throughput of the FP64 and FP32 pipes (bench support only,
// built as libd3d_peak.so, not part of the C ABI of libd3d_gb300).
//
// Each thread runs 8 independent FMA chains for `iters` rounds; the result is
// stored so the chains cannot be removed.  FLOP/s = 2 * 8 * iters * threads /
// seconds.
#include <cuda_runtime.h>

template <typename T>
__global__ void __launch_bounds__(256) k_fma(T* out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = (T)(threadIdx.x + k);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// Returns FLOP/s (FMA = 2), or a negative value on a CUDA error.
extern "C" double d3d_peak_fma_flops(int fp64, int iters, void* stream_) {
    cudaStream_t stream = reinterpret_cast<cudaStream_t>(stream_);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256, blocks = sms * 8;
    void* out = nullptr;
    if (cudaMallocAsync(&out, sizeof(double) * (size_t)blocks * threads, stream) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int rep = 0; rep < 2; ++rep) {  // the first launch warms up
        cudaEventRecord(e0, stream);
        if (fp64)
            k_fma<double><<<blocks, threads, 0, stream>>>(static_cast<double*>(out), iters, 0.999999, 1e-7);
        else
            k_fma<float><<<blocks, threads, 0, stream>>>(static_cast<float*>(out), iters, 0.999999f, 1e-7f);
        cudaEventRecord(e1, stream);
    }
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(out, stream);
    if (cudaStreamSynchronize(stream) != cudaSuccess || ms <= 0.f) return -1.0;
    return 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3);
}
