// FP64 / FP32 FMA throughput probe: independent FMA chains per thread.
#include <cstdio>
#include <cuda_runtime.h>
template <class T>
__global__ void fma_chain(T* out, int iters, T a, T b) {
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
template <class T> void run(const char* name, int blocks, int threads, int iters) {
    T* out; cudaMalloc(&out, sizeof(T) * blocks * threads);
    fma_chain<T><<<blocks, threads>>>(out, 16, (T)0.999, (T)0.001);
    cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
    cudaEventRecord(e0);
    fma_chain<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    float ms; cudaEventElapsedTime(&ms, e0, e1);
    double flops = 2.0 * 8 * (double)iters * blocks * threads;
    printf("%s: %.3f ms  %.2f TFLOP/s (FMA=2 flops) err=%s\n", name, ms, flops / ms / 1e9, cudaGetErrorString(cudaGetLastError()));
    cudaFree(out);
}
int main() {
    int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    printf("SMs %d\n", sms);
    run<double>("fp64", sms * 8, 256, 4096);
    run<float>("fp32", sms * 8, 256, 65536);
    return 0;
}
