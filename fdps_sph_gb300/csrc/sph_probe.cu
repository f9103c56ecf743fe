// FMA-throughput probe: the peak FP32 / FP64 CUDA-core rate of this GPU at
// its current clocks, measured with a register-resident chain of independent
// fused multiply-adds.  The pair kernels are bound by these pipes (no tensor
// cores: none of them is a contraction), so this is their roofline.
#include "sph_internal.cuh"

namespace {

template <class T, int CHAINS, int ITERS>
__global__ void k_fma_probe(T *out, T a, T b) {
    T acc[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) acc[c] = (T)(threadIdx.x + c);
    for (int it = 0; it < ITERS; ++it) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) acc[c] = acc[c] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += acc[c];
    if (s == (T)1.2345e-30) out[blockIdx.x] = s;   // keeps the chains live
}

}  // namespace

extern "C" int sph_probe_peak(int device, int fp64, double *tflops) {
    if (!tflops) return SPH_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    void *out = nullptr;
    if (cudaMalloc(&out, 1 << 20) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_OOM;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256;
    const int blocks = sms * 8;
    constexpr int CH = 8;
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
        float ms = 0.0f;
        double flops = 0.0;
        if (fp64) {
            constexpr int IT = 256;
            cudaEventRecord(e0);
            k_fma_probe<double, CH, IT><<<blocks, threads>>>((double *)out, 0.999999, 1e-7);
            cudaEventRecord(e1);
            flops = 2.0 * CH * IT * (double)threads * blocks;
        } else {
            constexpr int IT = 8192;
            cudaEventRecord(e0);
            k_fma_probe<float, CH, IT><<<blocks, threads>>>((float *)out, 0.999999f, 1e-7f);
            cudaEventRecord(e1);
            flops = 2.0 * CH * IT * (double)threads * blocks;
        }
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0.0f) best = fmax(best, flops / (ms * 1e-3) / 1e12);
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return SPH_ERR_CUDA;
    *tflops = best;
    return SPH_OK;
}
